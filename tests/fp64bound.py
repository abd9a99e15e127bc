"""The stated bound between FP32 vertices (GPU, reference operation order)
and the FP64 oracle's vertices of the same mesh.

Per vertex component:  |v32 - v64| <= 4 * ulp32(M),  M = max |coordinate| of
the volume's extent (max of |xyz_min|, |xyz_max| over the three axes).

Why ulp(M) and not ulp(|v|): every FP32 error term scales with the point
coordinates the vertex is interpolated from, not with the vertex itself, so a
vertex near 0 inside a volume that reaches 1023 carries errors of the size of
ulp(1023).  The worst-case rounding analysis (unit roundoff u = 2^-24, and
u * M < ulp(M)):
  ijk_to_xyz  (float)i/size*range + min (utils.hpp:118-122): <= 5 u M
  crossing    p0*(1-t) + p1*t, t = (iso-v0)/(v1-v0) (dmc.cu:1090-1098):
              <= 14 u M along the edge, <= 8 u M across it
  dual vertex sum of n <= 12 crossings in edge order, then / n
              (dmc.cu:1571-1592): + (n+1)/2 u M + u M
which gives at most 22 u M < 22 ulp(M).  Measured on the benchmark volumes
the largest error is 1.6 ulp(M) (64^3 sphere), 2.1 ulp(M) (512^3 blobs) and
2.6 ulp(M) (1024^3 uint16 noise; 1.6e-4 voxel), so the tested bound is 4.
"""
import numpy as np

K_ULP = 4.0


def extent_max(dims_xyz, xyz_min=None, xyz_max=None):
    mn = np.zeros(3) if xyz_min is None else np.abs(np.asarray(xyz_min, np.float64))
    mx = np.asarray(dims_xyz, np.float64) - 1 if xyz_max is None else np.abs(np.asarray(xyz_max, np.float64))
    return float(max(mn.max(), mx.max()))


def check(v32, v64, dims_xyz, xyz_min=None, xyz_max=None):
    """Assert the bound; return (max |d|, in ulps of M, in voxels)."""
    M = extent_max(dims_xyz, xyz_min, xyz_max)
    ulp = float(np.spacing(np.float32(M)))
    assert v32.shape == v64.shape
    if v32.size == 0:
        return 0.0, 0.0, 0.0
    d = np.abs(v32.astype(np.float64) - v64)
    worst = float(d.max())
    lo = np.zeros(3) if xyz_min is None else np.asarray(xyz_min, np.float64)
    hi = np.asarray(dims_xyz, np.float64) - 1 if xyz_max is None else np.asarray(xyz_max, np.float64)
    spacing = float(np.min(np.abs(hi - lo) / np.maximum(np.asarray(dims_xyz, np.float64) - 1, 1)))
    assert worst <= K_ULP * ulp, "FP32 vs FP64: %.3g > %g ulp(%g) = %.3g" % (worst, K_ULP, M, K_ULP * ulp)
    return worst, worst / ulp, worst / spacing
