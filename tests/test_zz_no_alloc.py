"""wtg_surfgreen_batch_noalloc: the allocation-free entry point.

It serves callers that cannot let this library allocate device memory (their
HBM is owned by another allocator's pool, or cudaMalloc's device-wide
synchronisation is not acceptable on their path).  Here it is called through
the C ABI on device buffers the test owns, twice in a row (the calls share the
library's fixed scratch), and each result must equal the allocating entry
point's within the FP64 parity tolerance used by every GPU test (1e-9
relative in dos_l / dos_r / dos_bulk; iteration counts and status equal).
"""
import ctypes as C

import numpy as np
import pytest

from wannier_tools_gb300 import _lib, api, synthetic

pytestmark = pytest.mark.gpu

EV = 1.0 / 27.211385
RTOL = 1e-9


def _colmajor(m):
    return np.asfortranarray(m).ravel(order="F")


def _run_case(lib, nw, np_, nk, omegas_ev, eta_ev, top, bot, seed):
    import torch
    m = synthetic.make_model(nw, np_, seed=seed)
    n = nw * np_
    kp = synthetic.random_kpoints(nk, seed=seed + 1)
    om = np.asarray(omegas_ev) * EV
    eta = eta_ev * EV
    with api.Model.from_surface_model(m) as g:
        ref = g.surface_spectrum(kp, om, eta, top, bot)
        hs = [g.ham_qlayer2qlayer(k) for k in kp]
    h = np.stack([np.stack([_colmajor(a), _colmajor(b)]) for a, b in hs])   # (nk, 2, n*n) complex
    dev = torch.device("cuda", 0)
    d_h = torch.from_numpy(np.ascontiguousarray(h).view(np.float64)).to(dev)
    d_om = torch.tensor(om, dtype=torch.float64, device=dev)
    nwo = len(om)
    top_a = np.asarray(top, np.int32)
    bot_a = np.asarray(bot, np.int32)
    ip = C.POINTER(C.c_int)
    for call in range(2):
        outs = [torch.full((nwo, nk), float("nan"), dtype=torch.float64, device=dev) for _ in range(3)]
        d_it = torch.full((nwo, nk), -1, dtype=torch.int32, device=dev)
        d_st = torch.full((nwo, nk), 255, dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        rc = lib.wtg_surfgreen_batch_noalloc(
            n, nw, nk, C.c_void_p(d_h.data_ptr()), nwo, C.c_void_p(d_om.data_ptr()), eta,
            api.ACCURACY_REF, api.ITERMAX_REF, len(top_a), top_a.ctypes.data_as(ip), len(bot_a),
            bot_a.ctypes.data_as(ip), 0, C.c_void_p(outs[0].data_ptr()), C.c_void_p(outs[1].data_ptr()),
            C.c_void_p(outs[2].data_ptr()), C.c_void_p(d_it.data_ptr()), C.c_void_p(d_st.data_ptr()), None)
        assert rc == _lib.WTG_OK, _lib.last_error()
        torch.cuda.synchronize()
        for name, t in zip(("dos_l", "dos_r", "dos_bulk"), outs):
            got = t.cpu().numpy().T                      # (nk, nomega)
            err = np.max(np.abs(got - ref[name]) / np.abs(ref[name]))
            assert err <= RTOL, (call, name, err)
        assert np.array_equal(d_it.cpu().numpy().T, ref["iters"]), call
        assert np.array_equal(d_st.cpu().numpy().T, ref["status"]), call


def test_noalloc_matches_allocating_entry_point(built_lib):
    _run_case(built_lib, 20, 2, 6, [-0.5, 0.0, 0.3], 1e-2, [1, 2, 5], [3, 20], seed=31)


def test_noalloc_scratch_caps_the_grid_ndim_112(built_lib):
    # 8 x 112^2 complex per CTA: the fixed scratch holds (64 MiB - 256 B) // (16 * 8 * 112^2) = 41
    # CTAs, fewer than the GPU's 152
    assert ((64 << 20) - 256) // (16 * 8 * 112 * 112) == 41
    _run_case(built_lib, 56, 2, 50, [0.0], 1e-3, list(range(1, 57)), list(range(1, 57)), seed=7)


def test_noalloc_rejects_sizes_beyond_its_limit(built_lib):
    # Ndim 200 is beyond the kernel's shared-memory limit (119); every buffer is
    # still a real allocation of the size the call describes.
    import torch
    n = 200
    dev = torch.device("cuda", 0)
    d_h = torch.zeros(2 * 2 * n * n, dtype=torch.float64, device=dev)
    d_om = torch.zeros(1, dtype=torch.float64, device=dev)
    outs = [torch.zeros(1, dtype=torch.float64, device=dev) for _ in range(3)]
    rc = built_lib.wtg_surfgreen_batch_noalloc(
        n, n, 1, C.c_void_p(d_h.data_ptr()), 1, C.c_void_p(d_om.data_ptr()), 1e-3, 1e-16, 100,
        0, None, 0, None, 0, C.c_void_p(outs[0].data_ptr()), C.c_void_p(outs[1].data_ptr()),
        C.c_void_p(outs[2].data_ptr()), None, None, None)
    torch.cuda.synchronize()
    assert rc == _lib.WTG_EUNSUPPORTED
    assert "exceeds" in _lib.last_error()
