"""dmc_extract_device_noalloc through the C ABI: two calls in a row, each
checked bit for bit against dmc_extract_device on the same input, with no
device memory allocated by either no-allocation call after the first.

The file name sorts last so that this runs after every other test; it also
passes on its own."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vol_struct(fg, t):
    dt = 0 if t.dtype.is_floating_point else 1
    return fg._volume_struct(t.data_ptr(), dt, (t.shape[2], t.shape[1], t.shape[0]))


def _outputs(torch, nv, nq):
    v = torch.full((max(nv, 1), 3), float("nan"), dtype=torch.float32, device="cuda")
    q = torch.full((max(nq, 1), 4), -1, dtype=torch.int32, device="cuda")
    t = torch.full((max(2 * nq, 1), 3), -1, dtype=torch.int32, device="cuda")
    return v, q, t


def _noalloc(fg, L, torch, t, mn, mx, iso, cap):
    vol = _vol_struct(fg, t)
    v, q, tr = _outputs(torch, *cap)
    nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = L.dmc_extract_device_noalloc(ctypes.byref(vol), fg._f3(mn), fg._f3(mx), ctypes.c_float(iso),
                                      v.data_ptr(), v.shape[0], q.data_ptr(), q.shape[0], tr.data_ptr(),
                                      ctypes.byref(nv), ctypes.byref(nq), None)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert rc == 0, fg.STATUS.get(rc, rc)
    nv, nq = nv.value, nq.value
    return (v[:nv].cpu().numpy(), q[:nq].cpu().numpy(), tr[:2 * nq].cpu().numpy()), free0 - free1


def _existing(fg, torch, ex, t, mn, mx, iso):
    nv, nq = ex.extract_device(t, mn, mx, iso)
    v, q, tr = _outputs(torch, nv, nq)
    ex.extract_device(t, mn, mx, iso, v, q, tr)
    torch.cuda.synchronize()
    return (v[:nv].cpu().numpy(), q[:nq].cpu().numpy(), tr[:2 * nq].cpu().numpy())


def _same(a, b):
    assert a[0].shape == b[0].shape and a[1].shape == b[1].shape
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_noalloc_two_calls_match_extract_device():
    import torch
    import framework_gb300 as fg
    from framework_gb300 import fields
    L = fg.load_library()
    cases = [
        (fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).cuda(), (0.0, 0.0, 0.0), (63.0, 63.0, 63.0), 0.0),
        (fields.value_noise_u16((97, 80, 70), base_period=16, seed=3).cuda(), (-1.0, 2.0, 0.5), (3.0, 5.0, 9.0),
         32768.0),
    ]
    with fg.Extractor(0, algo="simple") as ex:
        want = [_existing(fg, torch, ex, *c) for c in cases]
    grown = []
    for i, (t, mn, mx, iso) in enumerate(cases):
        cap = (len(want[i][0]), len(want[i][1]))
        got, grew = _noalloc(fg, L, torch, t, mn, mx, iso, cap)
        _same(got, want[i])
        grown.append(grew)
    # the second call runs entirely in memory that already existed
    assert grown[1] <= 2 << 20, "device free memory fell by %d bytes" % grown[1]


def test_noalloc_rejects_oversize_and_small_buffers():
    import torch
    import framework_gb300 as fg
    L = fg.load_library()
    assert 1024 * 1024 == fg.NOALLOC_MAX_CELLS
    t = torch.zeros((3, 1025, 1025), dtype=torch.float32, device="cuda")   # 2 x 1024 x 1024 cells
    vol = _vol_struct(fg, t)
    nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
    rc = L.dmc_extract_device_noalloc(ctypes.byref(vol), fg._f3((0, 0, 0)), fg._f3((1, 1, 1)), ctypes.c_float(0.5),
                                      None, 0, None, 0, None, ctypes.byref(nv), ctypes.byref(nq), None)
    assert fg.STATUS[rc] == "DMC_ERR_TOO_LARGE"
    # too-small buffers: overflow reported with the needed counts, context-free call stays usable
    from framework_gb300 import fields
    s = fields.sphere_sdf(32, radius=10.0, noise=0.0, seed=2).cuda()
    vol = _vol_struct(fg, s)
    v = torch.empty((4, 3), device="cuda")
    q = torch.empty((4, 4), dtype=torch.int32, device="cuda")
    rc = L.dmc_extract_device_noalloc(ctypes.byref(vol), fg._f3((0, 0, 0)), fg._f3((31, 31, 31)), ctypes.c_float(0.0),
                                      v.data_ptr(), 4, q.data_ptr(), 4, None, ctypes.byref(nv), ctypes.byref(nq), None)
    assert fg.STATUS[rc] == "DMC_ERR_OUTPUT_OVERFLOW" and nv.value > 4 and nq.value > 4
    rc = L.dmc_extract_device_noalloc(ctypes.byref(vol), fg._f3((0, 0, 0)), fg._f3((31, 31, 31)), ctypes.c_float(0.0),
                                      None, 0, None, 0, None, ctypes.byref(nv), ctypes.byref(nq), None)
    assert rc == 0 and nv.value > 4
