"""CPU oracle for the coated-sphere dn volume. TEST INFRASTRUCTURE ONLY.

Restates bpm/bpm/bpm_3d_spheres.py:create_dn_buffer (:11-38) with its kernel
bpm/bpm/kernels/bpm_3d_spheres.cl:fill_dn (:31-74) in numpy float32, every operation
rounded as the kernel writes it: r = (dx*i, dy*j, dz*k), the z-sorted centres between the
first with z >= r.z - rad2 and the last with z <= r.z + rad2, d = length(r - c) =
sqrt(((x^2 + y^2) + z^2) + 0), dmin starting at 1e9*rad2, dn = dn1 | dn2 | 0.
"""
import numpy as np


def create_dn_buffer(size, units, points, dn_inner=.0, rad_inner=0, dn_outer=.1, rad_outer=.4):
    """Restatement of create_dn_buffer (bpm/bpm/bpm_3d_spheres.py:11-38) and its kernel
    fill_dn (bpm/bpm/kernels/bpm_3d_spheres.cl:31-74), float32 with every operation rounded
    as the kernel writes it. Returns (Nz, Ny, Nx) float32."""
    Nx, Ny, Nz = size
    f = np.float32
    dx, dy, dz = (f(u) for u in units)
    ps = np.asarray(points, np.float64).reshape(-1, 3)
    ps = ps[np.argsort(ps[:, 2], kind="stable"), :].astype(np.float32)
    Np = ps.shape[0]
    rad1, rad2, dn1, dn2 = f(rad_inner), f(rad_outer), f(dn_inner), f(dn_outer)
    x = dx * np.arange(Nx, dtype=np.float32)
    y = dy * np.arange(Ny, dtype=np.float32)
    dn = np.zeros((Nz, Ny, Nx), np.float32)
    for k in range(Nz):
        z = dz * f(k)
        lo, hi = z - rad2, z + rad2
        ind1 = 0
        while ps[ind1, 2] < lo and ind1 < Np - 1:
            ind1 += 1
        ind2 = Np - 1
        while ps[ind2, 2] > hi and ind2 > 0:
            ind2 -= 1
        dmin = np.full((Ny, Nx), f(1000000000.) * rad2, np.float32)
        for n in range(ind1, ind2 + 1):
            ex = x - ps[n, 0]
            ey = y - ps[n, 1]
            ez = z - ps[n, 2]
            s = (ex * ex)[None, :] + (ey * ey)[:, None]
            s = s + f(ez * ez)
            s = s + f(0)
            d = np.sqrt(s, dtype=np.float32)
            dmin = np.where(d < dmin, d, dmin)
        dn[k] = np.where(dmin < rad2, np.where(dmin < rad1, dn1, dn2), f(0))
    return dn
