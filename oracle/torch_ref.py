"""FP64 torch restatement of the ignore-mode march, for gradients. TEST INFRASTRUCTURE ONLY
(the checker of the hand-written adjoint in tests/ and of bench.py's gradient figure).

The reference has no gradient; d(loss)/d(dn) of a march is checked against torch autograd
through this restatement of the per-step loop of bpm/bpm/bpm_3d.py:283-381 in mean mode
"ignore": u <- IFFT2(FFT2(u) * H) * exp(-i k0 dz dn[i+1]) * taper, with the FP64 propagator
and the FP32-recipe evanescent mask and taper of oracle.bpm_ref.
"""
import numpy as np

from . import bpm_ref


def march_exit_fp64(torch, dn, u0, size, units, lam, n0, absorbing_width=0):
    """Exit plane of the march of u0 (complex128 tensor, (..., Ny, Nx)) through dn (float64
    tensor, (Nz, Ny, Nx)); differentiable in both."""
    Nx, Ny, Nz = size
    dx, dy, dz = units
    k0 = 2 * np.pi / lam
    H, _ = bpm_ref.propagator_f64(n0, k0, dx, dy, dz, Nx, Ny)
    H = torch.as_tensor(H, device=dn.device)
    T = torch.as_tensor(bpm_ref.taper_f32(Nx, Ny, absorbing_width).astype(np.float64), device=dn.device)
    u = u0
    for i in range(Nz - 1):
        u = torch.fft.ifft2(torch.fft.fft2(u) * H)
        u = u * torch.exp(-1j * (k0 * dz) * dn[i + 1]) * T
    return u
