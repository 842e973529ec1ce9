"""Host-side mirror of the reference's surface-state interface over the C ABI.

Names and argument meaning follow the reference:

* ``Model.ham_qlayer2qlayer(k)``      -> (H00, H01)   src/ham_qlayer2qlayer.f90:1
* ``surfgreen_1985(omega, H00, H01, eta)`` -> (GLL, GRR, GB, iters, status)
                                                      src/surfgreen.f90:7
* ``Model.surface_spectrum(...)``     the (k, omega) loop bodies of surfstat
                                      (src/surfstat.f90:123-197) and
                                      SurfaceDOSkk (src/fermiarc.f90:206-248)
* ``surfstat`` / ``surface_dos_kk``   the drivers' grids, eta choice and output
                                      transforms (src/surfstat.f90:84-88,237-247;
                                      src/fermiarc.f90:68-70,140-150,193-194,372-397)

Error behaviour: the reference prints and continues on a failed zgesv and
silently stops at itermax; here each (k, omega) point carries a status
bitmask (PT_* flags) and hard errors raise ``WtgError``.  All computation of
the path runs in libwtgpu.so on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import PREC_FP64, PREC_MIXED, check  # noqa: F401

PI_REF = 3.14159265358979                    # src/module.f90:719
EV2HARTREE = 1.0 / 27.211385                 # src/module.f90:713
EPS9 = float(np.float32(1e-9))               # src/module.f90:728 (single-precision literal)
ACCURACY_REF = float(np.float32(1e-16))      # src/surfgreen.f90:42 (single-precision literal)
ITERMAX_REF = 100                            # src/surfgreen.f90:39
IJMAX_REF = 10                               # src/module.f90:505


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _from_colmajor(buf: np.ndarray, n: int) -> np.ndarray:
    """complex128 buffer of an n x n column-major matrix -> ndarray [i, j]."""
    return buf.reshape((n, n), order="F")


def _to_colmajor(m: np.ndarray) -> np.ndarray:
    return np.asfortranarray(m, dtype=np.complex128).ravel(order="F")


class Model:
    """A principal-layer model resident on the GPU (wtg_model_create)."""

    def __init__(self, hmnr: np.ndarray, irvec: np.ndarray, ndegen: np.ndarray | None,
                 np_: int, ijmax: int = IJMAX_REF):
        lib = _lib.load()
        hmnr = np.asarray(hmnr, dtype=np.complex128)
        nR, nw, nw2 = hmnr.shape
        if nw != nw2:
            raise ValueError("hmnr must have shape (nR, nw, nw)")
        # (nw, nw, nR) column-major == [R][j][i] row-major
        self._h = np.ascontiguousarray(hmnr.transpose(0, 2, 1))
        self._irv = np.ascontiguousarray(np.asarray(irvec, dtype=np.int32).reshape(nR, 3))
        self._nd = (np.ascontiguousarray(np.asarray(ndegen, dtype=np.int32))
                    if ndegen is not None else None)
        self.nw = nw
        self.np_ = int(np_)
        self.ijmax = int(ijmax)
        self.ndim = nw * self.np_
        handle = C.c_void_p()
        check(lib.wtg_model_create(nw, nR, _iptr(self._irv), _dptr(self._h.view(np.float64)),
                                   _iptr(self._nd) if self._nd is not None else None,
                                   self.np_, self.ijmax, C.byref(handle)))
        self._handle = handle

    @classmethod
    def from_surface_model(cls, m, ijmax: int = IJMAX_REF) -> "Model":
        return cls(m.hmnr, m.irvec, m.ndegen, m.np_, ijmax)

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            _lib.load().wtg_model_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_loto(self, born, diele=None, masses=None, cell_volume: float = 0.0):
        """Phonon LO-TO correction (ham_qlayer2qlayer_LOTO,
        src/ham_qlayer2qlayer.f90:312-476) for this model's Fourier sums.
        born: Born_Charge (natoms, 3, 3); diele: Diele_Tensor (3, 3); masses:
        Atom_Mass (natoms); cell_volume in the reference's units.  born=None
        switches it off."""
        lib = _lib.load()
        if born is None:
            check(lib.wtg_model_set_loto(self._handle, 0, None, None, None, 0.0))
            return
        z = np.asfortranarray(np.asarray(born, dtype=np.float64))
        d = np.asfortranarray(np.asarray(diele, dtype=np.float64))
        mm = np.ascontiguousarray(masses, dtype=np.float64)
        self._loto = (z, d, mm)
        check(lib.wtg_model_set_loto(self._handle, int(z.shape[0]), _dptr(z.ravel(order="F")),
                                     _dptr(d.ravel(order="F")), _dptr(mm), float(cell_volume)))

    # -- ham_qlayer2qlayer -------------------------------------------------
    def ham_qlayer2qlayer(self, k) -> tuple[np.ndarray, np.ndarray]:
        kk = np.ascontiguousarray(np.asarray(k, dtype=np.float64).reshape(2))
        n = self.ndim
        h00 = np.empty(n * n, dtype=np.complex128)
        h01 = np.empty(n * n, dtype=np.complex128)
        check(_lib.load().wtg_ham_qlayer2qlayer(self._handle, _dptr(kk), _dptr(h00.view(np.float64)),
                                                _dptr(h01.view(np.float64))))
        return _from_colmajor(h00, n), _from_colmajor(h01, n)

    # -- batched spectrum (host buffers) ------------------------------------
    def surface_spectrum(self, kpts, omegas, eta: float, top, bot,
                         tol: float = ACCURACY_REF, itermax: int = ITERMAX_REF,
                         divide_by_pi: bool = False, precision: int = PREC_FP64,
                         kcol=None, out: dict | None = None) -> dict:
        """dos_l / dos_r / dos_bulk / iters / status as (nk, nomega) arrays.

        ``kcol`` may give the k list already in the ABI layout (a contiguous
        (2, nk) float64 array, e.g. in pinned memory); ``out`` may give
        preallocated flat host arrays (dos_l, dos_r, dos_bulk float64,
        iters int32, status uint8, each nk*nomega long)."""
        if kcol is None:
            kp = np.asarray(kpts, dtype=np.float64).reshape(-1, 2)
            kcol = np.ascontiguousarray(kp.T)             # (nk, 2) column-major
        nk = kcol.shape[1]
        w = np.ascontiguousarray(np.asarray(omegas, dtype=np.float64).ravel())
        nwo = w.shape[0]
        top_a = np.ascontiguousarray(np.asarray(top, dtype=np.int32).ravel())
        bot_a = np.ascontiguousarray(np.asarray(bot, dtype=np.int32).ravel())
        if out is None:
            outs = {name: np.zeros(nk * nwo) for name in ("dos_l", "dos_r", "dos_bulk")}
            iters = np.zeros(nk * nwo, np.int32)
            status = np.zeros(nk * nwo, np.uint8)
        else:
            outs = {name: out[name] for name in ("dos_l", "dos_r", "dos_bulk")}
            iters = out["iters"]
            status = out["status"]
        check(_lib.load().wtg_surface_spectrum(
            self._handle, nk, _dptr(kcol), nwo, _dptr(w), float(eta), float(tol), int(itermax),
            len(top_a), _iptr(top_a), len(bot_a), _iptr(bot_a), int(bool(divide_by_pi)), precision,
            _dptr(outs["dos_l"]), _dptr(outs["dos_r"]), _dptr(outs["dos_bulk"]),
            iters.ctypes.data_as(C.POINTER(C.c_int32)), status.ctypes.data_as(C.POINTER(C.c_uint8))))
        res = {name: v.reshape((nk, nwo), order="F") for name, v in outs.items()}
        res["iters"] = iters.reshape((nk, nwo), order="F")
        res["status"] = status.reshape((nk, nwo), order="F")
        return res

    # -- spin-resolved spectrum (host buffers) ------------------------------
    def surface_spectrum_spin(self, kpts, omegas, eta: float, top, bot, arc: bool = False,
                              tol: float = ACCURACY_REF, itermax: int = ITERMAX_REF,
                              precision: int = PREC_FP64) -> dict:
        """surface_spectrum plus sx_l, sy_l, sz_l, sx_r, sy_r, sz_r ((nk, nomega)
        arrays): surfstat's spin sums (arc=False, src/surfstat.f90:162-192) or
        SurfaceDOSkk's spin texture (arc=True, src/fermiarc.f90:250-330)."""
        kp = np.asarray(kpts, dtype=np.float64).reshape(-1, 2)
        kcol = np.ascontiguousarray(kp.T)
        nk = kcol.shape[1]
        w = np.ascontiguousarray(np.asarray(omegas, dtype=np.float64).ravel())
        nwo = w.shape[0]
        top_a = np.ascontiguousarray(np.asarray(top, dtype=np.int32).ravel())
        bot_a = np.ascontiguousarray(np.asarray(bot, dtype=np.int32).ravel())
        outs = {name: np.zeros(nk * nwo) for name in ("dos_l", "dos_r", "dos_bulk")}
        spin = np.zeros(6 * nk * nwo)
        iters = np.zeros(nk * nwo, np.int32)
        status = np.zeros(nk * nwo, np.uint8)
        check(_lib.load().wtg_surface_spectrum_spin(
            self._handle, nk, _dptr(kcol), nwo, _dptr(w), float(eta), float(tol), int(itermax),
            len(top_a), _iptr(top_a), len(bot_a), _iptr(bot_a), int(bool(arc)), precision,
            _dptr(outs["dos_l"]), _dptr(outs["dos_r"]), _dptr(outs["dos_bulk"]), _dptr(spin),
            iters.ctypes.data_as(C.POINTER(C.c_int32)), status.ctypes.data_as(C.POINTER(C.c_uint8))))
        res = {name: v.reshape((nk, nwo), order="F") for name, v in outs.items()}
        for c, name in enumerate(("sx_l", "sy_l", "sz_l", "sx_r", "sy_r", "sz_r")):
            res[name] = spin[c * nk * nwo:(c + 1) * nk * nwo].reshape((nk, nwo), order="F")
        res["iters"] = iters.reshape((nk, nwo), order="F")
        res["status"] = status.reshape((nk, nwo), order="F")
        return res

    # -- batched spectrum (device buffers, asynchronous) --------------------
    def surface_spectrum_device(self, d_k, d_omega, eta: float, top, bot, d_dos_l, d_dos_r,
                                d_dos_bulk, d_iters=None, d_status=None,
                                tol: float = ACCURACY_REF, itermax: int = ITERMAX_REF,
                                divide_by_pi: bool = False, precision: int = PREC_FP64,
                                stream: int = 0) -> int:
        """Device-pointer form.  Arguments are torch CUDA tensors (or raw
        pointers via .data_ptr()): d_k (2, nk) row-major == (nk, 2) column-major,
        d_omega (nomega,), outputs (nomega, nk) row-major == (nk, nomega)
        column-major.  Enqueued on `stream` (a cudaStream_t value)."""
        nk = d_k.shape[1]
        nwo = d_omega.shape[0]
        top_a = np.ascontiguousarray(np.asarray(top, dtype=np.int32).ravel())
        bot_a = np.ascontiguousarray(np.asarray(bot, dtype=np.int32).ravel())

        def ptr(t):
            return None if t is None else C.c_void_p(t.data_ptr())

        return check(_lib.load().wtg_surface_spectrum_device(
            self._handle, nk, ptr(d_k), nwo, ptr(d_omega), float(eta), float(tol), int(itermax),
            len(top_a), _iptr(top_a), len(bot_a), _iptr(bot_a), int(bool(divide_by_pi)), precision,
            ptr(d_dos_l), ptr(d_dos_r), ptr(d_dos_bulk), ptr(d_iters), ptr(d_status),
            C.c_void_p(stream)))


    # -- tracing -------------------------------------------------------------
    def profile(self, enable: bool) -> None:
        """Reset and enable/disable per-launch CUDA-event timing (wtg_model_profile)."""
        check(_lib.load().wtg_model_profile(self._handle, int(enable)))

    def profile_read(self) -> dict:
        """Summed device ms of the Fourier and decimation launches since the
        last reset, and the number of this library's kernels launched."""
        f = C.c_double(0.0)
        d = C.c_double(0.0)
        n = C.c_longlong(0)
        nd = C.c_int(0)
        check(_lib.load().wtg_model_profile_read(self._handle, C.byref(f), C.byref(d), C.byref(n),
                                                 C.byref(nd)))
        return {"fourier_ms": f.value, "decim_ms": d.value, "launches": int(n.value),
                "decim_launches": int(nd.value)}

def _lists(models, tops, bots):
    ntop = np.ascontiguousarray([len(t) for t in tops], dtype=np.int32)
    nbot = np.ascontiguousarray([len(b) for b in bots], dtype=np.int32)
    top = np.ascontiguousarray(np.concatenate([np.asarray(t, np.int32) for t in tops] + [np.zeros(1, np.int32)]))
    bot = np.ascontiguousarray(np.concatenate([np.asarray(b, np.int32) for b in bots] + [np.zeros(1, np.int32)]))
    if len(tops) != len(models) or len(bots) != len(models):
        raise ValueError("one top and one bottom orbital list per model")
    return ntop, top, nbot, bot


def _points(point_model, kpts, omega, eta):
    pm = np.ascontiguousarray(point_model, dtype=np.int32).ravel()
    n = len(pm)
    kk = np.asarray(kpts, dtype=np.float64).reshape(n, 2)
    kcol = np.ascontiguousarray(kk.T).ravel()                  # (npts, 2) column-major
    om = np.ascontiguousarray(np.broadcast_to(np.asarray(omega, np.float64), (n,)))
    et = np.ascontiguousarray(np.broadcast_to(np.asarray(eta, np.float64), (n,)))
    return pm, kcol, om, et


class Engine:
    """A batch engine (wtg_engine_create): device tables of a fixed model set, a
    workspace for their largest Ndim and its own stream.  ``run`` solves points
    of several models (uneven Ndim, eta per point) in one persistent launch.
    One engine runs one batch at a time; separate engines run concurrently."""

    def __init__(self, models, tops, bots, precision: int = PREC_FP64, max_points: int = 4096,
                 graphs: bool | None = None):
        lib = _lib.load()
        self.models = list(models)
        self._ntop, self._top, self._nbot, self._bot = _lists(self.models, tops, bots)
        arr = (C.c_void_p * len(self.models))(*[m._handle.value for m in self.models])
        self._arr = arr
        h = C.c_void_p()
        check(lib.wtg_engine_create(len(self.models), arr, int(precision), int(max_points),
                                    _iptr(self._ntop), _iptr(self._top), _iptr(self._nbot),
                                    _iptr(self._bot), C.byref(h)))
        self._handle = h
        self.precision = int(precision)
        self.max_points = int(max_points)
        if graphs is not None:
            check(lib.wtg_engine_set_graphs(h, 1 if graphs else 0))

    def set_graphs(self, on: bool):
        """Replay runs from captured CUDA graphs (default) or launch them directly."""
        check(_lib.load().wtg_engine_set_graphs(self._handle, 1 if on else 0))

    def graph_info(self) -> dict:
        g = C.c_int(0)
        n = C.c_longlong(0)
        check(_lib.load().wtg_engine_graph_info(self._handle, C.byref(g), C.byref(n)))
        return {"graphs": int(g.value), "graph_launches": int(n.value)}

    def info(self) -> dict:
        b = C.c_longlong(0)
        mp = C.c_int(0)
        la = C.c_longlong(0)
        check(_lib.load().wtg_engine_info(self._handle, C.byref(b), C.byref(mp), C.byref(la)))
        return {"device_bytes": int(b.value), "max_points": int(mp.value), "launches": int(la.value)}

    def run(self, point_model, kpts, omega, eta, tol: float = ACCURACY_REF,
            itermax: int = ITERMAX_REF, divide_by_pi: bool = False) -> dict:
        """Per point: dos_l, dos_r, dos_bulk, iters, status (arrays of npts)."""
        pm, kcol, om, et = _points(point_model, kpts, omega, eta)
        n = len(pm)
        out = {name: np.empty(n, np.float64) for name in ("dos_l", "dos_r", "dos_bulk")}
        out["iters"] = np.empty(n, np.int32)
        out["status"] = np.empty(n, np.uint8)
        check(_lib.load().wtg_engine_run(
            self._handle, n, _iptr(pm), _dptr(kcol), _dptr(om), _dptr(et), float(tol), int(itermax),
            1 if divide_by_pi else 0, _dptr(out["dos_l"]), _dptr(out["dos_r"]), _dptr(out["dos_bulk"]),
            out["iters"].ctypes.data_as(C.POINTER(C.c_int32)),
            out["status"].ctypes.data_as(C.POINTER(C.c_uint8))))
        return out

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            _lib.load().wtg_engine_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def set_tile(precision: int, ndim: int, value: int) -> None:
    """Launch shape used at this Ndim (wtg_tile_set): FP64 threads per CTA, mixed pass
    width; 0 restores the built-in choice."""
    check(_lib.load().wtg_tile_set(int(precision), int(ndim), int(value)))


def get_tile(precision: int, ndim: int) -> tuple[int, int]:
    """(value in use, built-in value) at this Ndim (wtg_tile_get)."""
    v = C.c_int(0)
    b = C.c_int(0)
    check(_lib.load().wtg_tile_get(int(precision), int(ndim), C.byref(v), C.byref(b)))
    return int(v.value), int(b.value)


def batch_spectrum(models, tops, bots, point_model, kpts, omega, eta, tol: float = ACCURACY_REF,
                   itermax: int = ITERMAX_REF, divide_by_pi: bool = False,
                   precision: int = PREC_FP64) -> dict:
    """One uneven batch (wtg_batch_spectrum): point p of model point_model[p]
    at kpts[p], omega[p], eta[p] (Hartree); per-point outputs."""
    models = list(models)
    ntop, top, nbot, bot = _lists(models, tops, bots)
    pm, kcol, om, et = _points(point_model, kpts, omega, eta)
    n = len(pm)
    out = {name: np.empty(n, np.float64) for name in ("dos_l", "dos_r", "dos_bulk")}
    out["iters"] = np.empty(n, np.int32)
    out["status"] = np.empty(n, np.uint8)
    arr = (C.c_void_p * len(models))(*[m._handle.value for m in models])
    check(_lib.load().wtg_batch_spectrum(
        len(models), arr, n, _iptr(pm), _dptr(kcol), _dptr(om), _dptr(et), float(tol), int(itermax),
        _iptr(ntop), _iptr(top), _iptr(nbot), _iptr(bot), 1 if divide_by_pi else 0, int(precision),
        _dptr(out["dos_l"]), _dptr(out["dos_r"]), _dptr(out["dos_bulk"]),
        out["iters"].ctypes.data_as(C.POINTER(C.c_int32)),
        out["status"].ctypes.data_as(C.POINTER(C.c_uint8))))
    return out


def surfgreen_1985(omega: float, h00: np.ndarray, h01: np.ndarray, eta: float,
                   tol: float = ACCURACY_REF, itermax: int = ITERMAX_REF):
    """One decimation on the GPU: (GLL, GRR, GB, iters, status)."""
    n = h00.shape[0]
    a = _to_colmajor(h00)
    b = _to_colmajor(h01)
    gll = np.empty(n * n, np.complex128)
    grr = np.empty(n * n, np.complex128)
    gb = np.empty(n * n, np.complex128)
    it = C.c_int(0)
    st = C.c_int(0)
    check(_lib.load().wtg_surfgreen_1985(n, float(omega), float(eta), _dptr(a.view(np.float64)),
                                         _dptr(b.view(np.float64)), float(tol), int(itermax),
                                         _dptr(gll.view(np.float64)), _dptr(grr.view(np.float64)),
                                         _dptr(gb.view(np.float64)), C.byref(it), C.byref(st)))
    return (_from_colmajor(gll, n), _from_colmajor(grr, n), _from_colmajor(gb, n),
            int(it.value), int(st.value))


def mat_mul(a: np.ndarray, b: np.ndarray, precision: int = PREC_FP64) -> np.ndarray:
    """C = A*B on the GPU (mat_mul, src/mat_mul.f90:3-27)."""
    n = a.shape[0]
    x = _to_colmajor(a)
    y = _to_colmajor(b)
    c = np.empty(n * n, np.complex128)
    check(_lib.load().wtg_mat_mul(n, _dptr(x.view(np.float64)), _dptr(y.view(np.float64)),
                                  _dptr(c.view(np.float64)), precision))
    return _from_colmajor(c, n)


def inv(a: np.ndarray, precision: int = PREC_FP64):
    """A^-1 on the GPU (inv, src/inverse.f90:1-58): (inverse, status)."""
    n = a.shape[0]
    x = _to_colmajor(a).copy()
    st = C.c_int(0)
    check(_lib.load().wtg_inv(n, _dptr(x.view(np.float64)), precision, C.byref(st)))
    return _from_colmajor(x, n), int(st.value)


def device_info() -> str:
    buf = C.create_string_buffer(256)
    check(_lib.load().wtg_device_info(buf, 256))
    return buf.value.decode()


# --- driver-level helpers (grids and output transforms of the reference) ----

def surfstat_grid(omegamin: float, omegamax: float, omeganum: int):
    """src/surfstat.f90:84-88: eta = 3 (wmax - wmin)/nw; omega excludes wmax."""
    eta = (omegamax - omegamin) / float(omeganum) * 3.0
    omega = np.array([omegamin + (i - 1) * (omegamax - omegamin) / float(omeganum)
                      for i in range(1, omeganum + 1)])
    return omega, eta


def kpath_slab(lines, nk: int) -> np.ndarray:
    """k2_path of src/readinput.f90:2180-2195: nk points per line (endpoints
    included, so segment ends repeat); ``lines`` = [(kstart(2), kend(2)), ...]."""
    out = np.zeros((nk * len(lines), 2))
    for j, (ks, ke) in enumerate(lines):
        ks = np.asarray(ks, float)
        ke = np.asarray(ke, float)
        for i in range(1, nk + 1):
            out[i - 1 + j * nk] = ks + (ke - ks) * (i - 1) / float(nk - 1)
    return out


def kplane_slab(nk1: int, nk2: int, k2d_start, vec1, vec2):
    """src/fermiarc.f90:68-70,140-150: nkx, nky bumped to odd; returns
    (nkx, nky, k12[(nkx*nky), 2]) with the j (second) index fastest."""
    nkx = nk1 + 1 if nk1 % 2 == 0 else nk1
    nky = nk2 + 1 if nk2 % 2 == 0 else nk2
    i = np.repeat(np.arange(nkx), nky).astype(float)
    j = np.tile(np.arange(nky), nkx).astype(float)
    s = np.asarray(k2d_start, float)
    v1 = np.asarray(vec1, float)
    v2 = np.asarray(vec2, float)
    k12 = np.stack([s[c] + i * v1[c] / float(nkx - 1) + j * v2[c] / float(nky - 1) for c in range(2)], 1)
    return nkx, nky, k12


def surfstat(model: Model, k2_path, omegamin: float, omegamax: float, omeganum: int, top, bot,
             tol: float = ACCURACY_REF, itermax: int = ITERMAX_REF, particle: str = "electron") -> dict:
    """surfstat (src/surfstat.f90:1-260) without file output: returns raw
    sums plus the written quantities log|dos| and *_only.  For phonons the
    omega grid is squared after eta is set (src/surfstat.f90:90-96)."""
    omega, eta = surfstat_grid(omegamin, omegamax, omeganum)
    if "phonon" in particle:
        omega = omega * omega
    r = model.surface_spectrum(k2_path, omega, eta, top, bot, tol, itermax, divide_by_pi=False)
    r["omega"] = omega
    r["eta"] = eta
    r.update(surfstat_post(r["dos_l"], r["dos_r"], r["dos_bulk"]))
    return r


def surface_dos_kk(model: Model, nk1: int, nk2: int, k2d_start, vec1, vec2, iso_energy: float,
                   fermi_broadening: float, top, bot, tol: float = ACCURACY_REF,
                   itermax: int = ITERMAX_REF, particle: str = "electron") -> dict:
    """SurfaceDOSkk arc maps (src/fermiarc.f90:1-460) without file output.
    For phonons the energy is squared (src/fermiarc.f90:196-200); the LO-TO
    form follows Model.set_loto."""
    nkx, nky, k12 = kplane_slab(nk1, nk2, k2d_start, vec1, vec2)
    if "phonon" in particle:
        iso_energy = iso_energy * iso_energy
    r = model.surface_spectrum(k12, [iso_energy], fermi_broadening, top, bot, tol, itermax,
                               divide_by_pi=True)
    out = {name: r[name][:, 0].reshape(nkx, nky) for name in ("dos_l", "dos_r", "dos_bulk", "iters", "status")}
    out["k12"] = k12
    l_only, r_only = arc_post(out["dos_l"], out["dos_r"])
    out["dos_l_only"] = l_only
    out["dos_r_only"] = r_only
    return out


def surfstat_post(dos_l, dos_r, dos_bulk) -> dict:
    """src/surfstat.f90:237-247."""
    l_only = dos_l - dos_bulk
    l_only = np.where(l_only < 0, EPS9, l_only)
    r_only = dos_r - dos_bulk
    r_only = np.where(r_only < 0, EPS9, r_only)
    return {"log_dos_l": np.log(np.abs(dos_l)), "log_dos_r": np.log(np.abs(dos_r)),
            "log_dos_bulk": np.log(np.abs(dos_bulk) + EPS9), "dos_l_only": l_only,
            "dos_r_only": r_only}


def arc_post(dos_l, dos_r):
    """src/fermiarc.f90:372-397."""
    return (np.where(dos_l < dos_l.max() / 10.0, EPS9, dos_l),
            np.where(dos_r < dos_r.max() / 10.0, EPS9, dos_r))


def jdos_kpath(dos) -> np.ndarray:
    """surfstat's joint DOS along the k path (src/surfstat.f90:889-905):
    dos[nk, nomega] -> jdos[nk, nomega], on the GPU."""
    d = np.asfortranarray(np.asarray(dos, dtype=np.float64))
    nk, nom = d.shape
    out = np.empty((nk, nom), dtype=np.float64, order="F")
    check(_lib.load().wtg_jdos_kpath(nk, nom, _dptr(d), _dptr(out)))
    return out


def qpi_kplane(chans, p1: int | None = None, p2: int | None = None, scale: float | None = None):
    """QPI on the k plane (src/fermiarc.f90:497-545) on the GPU.  chans: one
    (nkx, nky) array (jdos of dos_*_only) or four (dos_only, sx, sy, sz: the
    spin form).  Periods default to nkx-1, nky-1; scale to 1/(nkx*nky) for one
    channel and 1 for four, as the reference.  Returns jdos[nkx*nky] in ikp
    order (second index fastest)."""
    arrs = [np.asarray(c, dtype=np.float64) for c in (chans if isinstance(chans, (list, tuple)) else [chans])]
    nkx, nky = arrs[0].shape
    buf = np.concatenate([np.asfortranarray(a).ravel(order="F") for a in arrs])
    p1 = nkx - 1 if p1 is None else int(p1)
    p2 = nky - 1 if p2 is None else int(p2)
    if scale is None:
        scale = 1.0 / (nkx * nky) if len(arrs) == 1 else 1.0
    out = np.empty(nkx * nky, dtype=np.float64)
    check(_lib.load().wtg_jdos_kplane(nkx, nky, p1, p2, len(arrs), _dptr(buf), float(scale), _dptr(out)))
    return out


def fp64_peak_tflops() -> float:
    """FP64 DFMA throughput of the current GPU (wtg_probe_fp64_peak)."""
    v = C.c_double(0.0)
    check(_lib.load().wtg_probe_fp64_peak(C.byref(v)))
    return float(v.value)


def dmma_peak_tflops() -> float:
    """FP64 tensor-core (DMMA) throughput of the current GPU (wtg_probe_dmma_peak)."""
    v = C.c_double(0.0)
    check(_lib.load().wtg_probe_dmma_peak(C.byref(v)))
    return float(v.value)

