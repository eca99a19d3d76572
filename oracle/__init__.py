"""CPU oracle for the bpm_gb300 hot paths. TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may import
this package, and only as the checker (or the timed CPU baseline); the product
path in bpm_gb300/ never imports it.

Modules:
  bpm_ref    -- numpy restatement of the split-step z-march of bpm/bpm/bpm_3d.py
                (_bpm_3d, _bpm_3d_split) and of the Bpm3d class path
                (bpm/bpmclass/bpm3d.py, bpm/bpmclass/_bpm3d_ocl.py), in a
                reference-faithful FP32 flavour and an FP64 flavour.
  debye_ref  -- numpy restatement of focus_field_debye / psf / psf_u0
                (bpm/psf/_focus_fields_debye.py, bpm/psf/kernels/psf_debye.cl,
                bpm/psf/psf_functions.py) in FP64 with scipy Bessel functions.
  torch_ref  -- FP64 torch restatement of the ignore-mode march (autograd reference
                for the adjoint's gradient).
  reflib     -- ctypes loader for oracle/_ref/libref_cl.so, the reference's own
                OpenCL kernel sources compiled as host C++ (built by oracle/Makefile
                where the reference checkout exists; absent elsewhere).
"""
