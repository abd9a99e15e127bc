"""dmc_extract_device_noalloc through the C ABI.

This entry point is for callers that cannot let the library allocate device
memory: a process whose free device memory is reserved by its own pool
allocator, or a latency-bound loop where cudaMalloc/cudaFree would
synchronise the device.  Its scratch is one fixed array in the library's
module memory.

Checked here, each call bit for bit against the CPU oracle and against
dmc_extract_device on the same input:
  * two calls in a row, the second allocating no device memory;
  * a volume of exactly DMC_NOALLOC_MAX_CELLS cells, and the first size past it;
  * the first call of a fresh process made on a non-blocking stream (the
    table upload of the set-up must be complete before that stream's kernels).

The file name sorts last so that this runs after every other test; it also
passes on its own."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _vol_struct(fg, t):
    dt = 0 if t.dtype.is_floating_point else 1
    return fg._volume_struct(t.data_ptr(), dt, (t.shape[2], t.shape[1], t.shape[0]))


def _outputs(torch, nv, nq):
    v = torch.full((max(nv, 1), 3), float("nan"), dtype=torch.float32, device="cuda")
    q = torch.full((max(nq, 1), 4), -1, dtype=torch.int32, device="cuda")
    t = torch.full((max(2 * nq, 1), 3), -1, dtype=torch.int32, device="cuda")
    return v, q, t


def _noalloc(fg, L, torch, t, mn, mx, iso, cap, stream=None):
    vol = _vol_struct(fg, t)
    v, q, tr = _outputs(torch, *cap)
    nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = L.dmc_extract_device_noalloc(ctypes.byref(vol), fg._f3(mn), fg._f3(mx), ctypes.c_float(iso),
                                      v.data_ptr(), v.shape[0], q.data_ptr(), q.shape[0], tr.data_ptr(),
                                      ctypes.byref(nv), ctypes.byref(nq),
                                      None if stream is None else ctypes.c_void_p(stream.cuda_stream))
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


def _oracle(t, mn, mx, iso):
    import oracle
    from framework_gb300 import fields
    import torch
    a = fields.as_u16_numpy(t) if t.dtype == torch.int16 else t.cpu().numpy()
    r = oracle.extract(a, mn, mx, iso)
    return (r["vertices"], r["quads"].astype(np.int32), r["triangles"].astype(np.int32))


def _same(a, b):
    """Vertices bit for bit (tolerance zero), quads and triangles equal."""
    assert a[0].shape == b[0].shape and a[1].shape == b[1].shape
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def _cases(torch):
    from framework_gb300 import fields
    return [
        (fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).cuda(), (0.0, 0.0, 0.0), (63.0, 63.0, 63.0), 0.0),
        (fields.value_noise_u16((97, 80, 70), base_period=16, seed=3).cuda(), (-1.0, 2.0, 0.5), (3.0, 5.0, 9.0),
         32768.0),
    ]


def test_noalloc_two_calls_match_oracle_and_extract_device():
    import torch
    import framework_gb300 as fg
    L = fg.load_library()
    cases = _cases(torch)
    with fg.Extractor(0, algo="simple") as ex:
        want = [_existing(fg, torch, ex, *c) for c in cases]
    grown = []
    for i, c in enumerate(cases):
        _same(want[i], _oracle(*c))
        cap = (len(want[i][0]), len(want[i][1]))
        got, grew = _noalloc(fg, L, torch, *c, cap)
        _same(got, want[i])
        grown.append(grew)
    # the second call runs entirely in memory that already existed
    assert grown[1] <= 2 << 20, "device free memory fell by %d bytes" % grown[1]


def test_noalloc_at_the_cell_limit():
    """1025 x 1025 x 2 points = exactly DMC_NOALLOC_MAX_CELLS cells: accepted and
    equal to the oracle; one more row of cells is rejected before any GPU work."""
    import torch
    import framework_gb300 as fg
    from framework_gb300 import fields
    L = fg.load_library()
    assert 1024 * 1024 == fg.NOALLOC_MAX_CELLS
    t = fields.value_noise_u16((1025, 1025, 2), base_period=32, seed=11).cuda()
    mn, mx, iso = (0.0, 0.0, 0.0), (1024.0, 1024.0, 1.0), 32768.0
    want = _oracle(t, mn, mx, iso)
    got, _ = _noalloc(fg, L, torch, t, mn, mx, iso, (len(want[0]), len(want[1])))
    _same(got, want)
    big = torch.zeros((2, 1026, 1025), dtype=torch.int16, device="cuda")   # 1024 x 1025 x 1 cells
    vol = _vol_struct(fg, big)
    nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
    rc = L.dmc_extract_device_noalloc(ctypes.byref(vol), fg._f3(mn), fg._f3(mx), ctypes.c_float(iso),
                                      None, 0, None, 0, None, ctypes.byref(nv), ctypes.byref(nq), None)
    assert fg.STATUS[rc] == "DMC_ERR_TOO_LARGE"


_FIRST_CALL_ON_SIDE_STREAM = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, %r)
import framework_gb300 as fg
from framework_gb300 import fields
import oracle
L = fg.load_library()
t = fields.sphere_sdf(48, radius=15.0, noise=0.01, seed=4).cuda()
want = oracle.extract(t.cpu().numpy(), iso=0.0)
nv0, nq0 = len(want["vertices"]), len(want["quads"])
s = torch.cuda.Stream()          # created non-blocking: not ordered after the legacy default stream
v = torch.full((nv0, 3), float("nan"), device="cuda")
q = torch.full((nq0, 4), -1, dtype=torch.int32, device="cuda")
torch.cuda.synchronize()
vol = fg._volume_struct(t.data_ptr(), 0, (48, 48, 48))
nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
rc = L.dmc_extract_device_noalloc(ctypes.byref(vol), fg._f3((0, 0, 0)), fg._f3((47, 47, 47)), ctypes.c_float(0.0),
                                  v.data_ptr(), nv0, q.data_ptr(), nq0, None, ctypes.byref(nv), ctypes.byref(nq),
                                  ctypes.c_void_p(s.cuda_stream))
torch.cuda.synchronize()
assert rc == 0, rc
assert (nv.value, nq.value) == (nv0, nq0)
assert np.array_equal(v.cpu().numpy().view(np.uint32), want["vertices"].view(np.uint32))
assert np.array_equal(q.cpu().numpy().astype(np.uint32), want["quads"])
print("first call on a side stream ok")
"""


def test_noalloc_first_call_on_non_blocking_stream():
    """A fresh process whose first call runs on a stream created non-blocking."""
    r = subprocess.run([sys.executable, "-c", _FIRST_CALL_ON_SIDE_STREAM % ROOT], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "first call on a side stream ok" in r.stdout


def test_noalloc_rejects_oversize_and_small_buffers():
    import torch
    import framework_gb300 as fg
    L = fg.load_library()
    t = torch.zeros((3, 1025, 1025), dtype=torch.float32, device="cuda")   # 2 x 1024 x 1024 cells
    vol = _vol_struct(fg, t)
    nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
    rc = L.dmc_extract_device_noalloc(ctypes.byref(vol), fg._f3((0, 0, 0)), fg._f3((1, 1, 1)), ctypes.c_float(0.5),
                                      None, 0, None, 0, None, ctypes.byref(nv), ctypes.byref(nq), None)
    assert fg.STATUS[rc] == "DMC_ERR_TOO_LARGE"
    # dims whose cell count overflows 64 bits are rejected, not wrapped
    huge = fg._volume_struct(t.data_ptr(), 0, (0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF))
    rc = L.dmc_extract_device_noalloc(ctypes.byref(huge), fg._f3((0, 0, 0)), fg._f3((1, 1, 1)), ctypes.c_float(0.5),
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
