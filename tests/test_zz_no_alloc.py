"""The allocation-free step kr_step_static against kr_step, through the C ABI.

kr_step_static keeps its Krylov workspace in a fixed array inside the library,
so callers that may not allocate device memory when they step (code recorded
into CUDA graphs, hosts whose device memory belongs to their own pool
allocator) can still propagate. Its results must equal kr_step's, call after
call, although the array keeps the previous call's contents. This file is
collected last on purpose; it passes alone in a fresh process and after the
other tests."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

STATE_RTOL = 1e-10  # per-step state tolerance of the GPU parity tests


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _call(entry, plan, v, phase, fac, korder):
    from richmol_gb300 import _native
    from richmol_gb300.device import stream_ptr
    rc = entry(plan.op, v.data_ptr(), v.shape[0], phase.data_ptr(), float(fac.real), float(fac.imag), 1e-15, 0,
               korder.ctypes.data, stream_ptr())
    _native.check(rc, plan.ctx)


@pytest.mark.parametrize("products", ["f64", "df"])
def test_static_scratch_step_matches_kr_step_twice(products):
    from richmol_gb300 import CarTens, TDSE, _native
    if not os.path.exists(_native.LIB_PATH):
        _native.build_library()
    L = _native.lib()
    from oracle import fixtures
    path = os.path.join(GOLDEN, "asym_j4.npz")
    d, meta = fixtures.load(path)
    sc = meta["scales"]
    h0 = CarTens(path, name="h0")
    Hdc = (CarTens(path, name="dip") * meta["dc"]) * sc["dc"]
    Hac = CarTens(path, name="pol") * sc["ac"]
    td = TDSE(t_start=0.9, t_end=1.0, dt=0.005)
    td.time_grid()
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    a = torch.from_numpy(v0.copy()).cuda()
    b = torch.from_numpy(v0.copy()).cuda()
    phase = td._h0_phase(h0, td.exp_fac, a.device)
    for i in range(2):  # two calls in a row: the array keeps the previous call's contents
        Hac.field(d["split/fields"][i])
        plan = (Hdc + Hac).device_operator()
        plan.set_precision(products)  # the static step has the double-float copy of x in its array too
        ka = np.zeros(a.shape[0], np.int32)
        kb = np.zeros(b.shape[0], np.int32)
        _call(L.kr_step, plan, a, phase, td.exp_fac, ka)
        _call(L.kr_step_static, plan, b, phase, td.exp_fac, kb)
        torch.cuda.synchronize()
        assert np.array_equal(ka, kb)
        assert np.array_equal(b.cpu().numpy(), a.cpu().numpy())  # the same kernel, bit for bit
    # and it follows the reference's own propagation
    ref = d["split/states_first2"][1]
    assert _rel(b.cpu().numpy()[:2], ref) < STATE_RTOL
    plan.set_precision("f64")


def test_product_precision_argument_checked():
    from richmol_gb300 import CarTens, _native
    from oracle import fixtures
    path = os.path.join(GOLDEN, "asym_j4.npz")
    d, meta = fixtures.load(path)
    Hac = CarTens(path, name="pol") * meta["scales"]["ac"]
    Hac.field(d["split/fields"][0])
    plan = Hac.device_operator()
    with pytest.raises(ValueError):
        plan.set_precision("f32")
    assert _native.lib().kr_op_set_precision(plan.op, 7) == _native.KR_ERR_ARG
    plan.set_precision("df")
    plan.set_precision("f64")


def test_static_scratch_rejects_oversized_operator():
    from richmol_gb300 import _native, workloads
    L = _native.lib()
    wl = workloads.asym_top(Jmax=32)  # dim 47,905: about 80 MB of workspace at maxorder 100
    wl.Hac.field([0.0, 0.0, 1e9])
    plan = wl.Hac.device_operator()
    need, cap = ctypes.c_size_t(), ctypes.c_size_t()
    assert L.kr_static_scratch_bytes(plan.op, ctypes.byref(need), ctypes.byref(cap)) == 0
    assert need.value > cap.value == 64 << 20
    v = torch.zeros((1, wl.dim), dtype=torch.complex128, device="cuda")
    v[0, 0] = 1.0
    before = v.clone()
    from richmol_gb300.device import stream_ptr
    rc = L.kr_step_static(plan.op, v.data_ptr(), 1, None, 0.0, -1e-3, 1e-15, 0, None, stream_ptr())
    assert rc == _native.KR_ERR_ARG
    assert "static scratch holds" in _native.last_error(plan.ctx)
    torch.cuda.synchronize()
    assert torch.equal(v, before)


def _asym_setup():
    from oracle import fixtures
    from richmol_gb300 import CarTens, TDSE
    path = os.path.join(GOLDEN, "asym_j4.npz")
    d, meta = fixtures.load(path)
    sc = meta["scales"]
    h0 = CarTens(path, name="h0")
    Hdc = (CarTens(path, name="dip") * meta["dc"]) * sc["dc"]
    Hac = CarTens(path, name="pol") * sc["ac"]
    td = TDSE(t_start=0.9, t_end=1.0, dt=0.005)
    td.time_grid()
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    Hac.field(d["split/fields"][0])
    return td, h0, Hdc + Hac, v0


def _call_nosync(entry, plan, v, phase, fac):
    from richmol_gb300 import _native
    from richmol_gb300.device import stream_ptr
    rc = entry(plan.op, v.data_ptr(), v.shape[0], phase.data_ptr(), float(fac.real), float(fac.imag), 1e-15, 0,
               None, stream_ptr())
    _native.check(rc, plan.ctx)


def test_static_scratch_step_recorded_in_a_graph_matches_kr_step():
    """korder == NULL (no host read-back): the call can be recorded into a CUDA
    graph once the first call on the device has looked up the array; two
    replays equal two kr_step calls, and the status hand-off reports no error."""
    from richmol_gb300 import _native
    L = _native.lib()
    td, h0, H, v0 = _asym_setup()
    plan = H.device_operator()
    a = torch.from_numpy(v0.copy()).cuda()
    b = torch.from_numpy(v0.copy()).cuda()
    warm = torch.from_numpy(v0.copy()).cuda()
    phase = td._h0_phase(h0, td.exp_fac, a.device)
    dev_before = torch.cuda.current_device()
    _call_nosync(L.kr_step_static, plan, warm, phase, td.exp_fac)  # set-up call, outside the recording
    assert torch.cuda.current_device() == dev_before
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.graph(g, stream=s):
        _call_nosync(L.kr_step_static, plan, b, phase, td.exp_fac)
    torch.cuda.current_stream().wait_stream(s)
    for _ in range(2):
        g.replay()
        _call_nosync(L.kr_step, plan, a, phase, td.exp_fac)
    torch.cuda.synchronize()
    plan.sync_status()
    assert _rel(b.cpu().numpy(), a.cpu().numpy()) < STATE_RTOL


def test_static_scratch_step_maxorder_reported_and_pending_error_kept():
    """A Lanczos that cannot converge within maxorder: with korder == NULL the
    error reaches kr_sync_status; while it is pending, a further call skips its
    work and reports it (as kr_step does), after which the status is clear."""
    from richmol_gb300 import _native
    L = _native.lib()
    td, h0, H, v0 = _asym_setup()
    plan = H.device_operator(maxorder=3)
    phase = td._h0_phase(h0, td.exp_fac, torch.device("cuda"))
    v = torch.from_numpy(v0.copy()).cuda()
    _call_nosync(L.kr_step_static, plan, v, phase, td.exp_fac)
    with pytest.raises(_native.KrylovError) as ei:
        plan.sync_status()
    assert ei.value.code == _native.KR_ERR_MAXORDER
    plan.sync_status()  # reported once, then clear
    # an error left pending by a call without read-back ...
    _call_nosync(L.kr_step_static, plan, v, phase, td.exp_fac)
    torch.cuda.synchronize()
    before = v.clone()
    # ... makes the next call skip its work and report that error
    from richmol_gb300.device import stream_ptr
    kord = np.zeros(v.shape[0], np.int32)
    rc = L.kr_step_static(plan.op, v.data_ptr(), v.shape[0], phase.data_ptr(), float(td.exp_fac.real),
                          float(td.exp_fac.imag), 1e-15, 0, kord.ctypes.data, stream_ptr())
    assert rc == _native.KR_ERR_MAXORDER
    torch.cuda.synchronize()
    assert torch.equal(v, before)
    plan.sync_status()  # the read-back call took the error over
