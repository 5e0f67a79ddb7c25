"""ctypes binding of the C ABI (include/fdfk_gb300.h) with the reference's array conventions.

Arrays are numpy arrays in Fortran order with the shapes the reference
allocates (src/FDFK2D.f90:253-355):

* ``c``: ``(3, nz+npml, nx+2*npml)`` = rho, lambda, mu (src/FDFK2D.f90:125)
* ``ux``, ``uz``: ``(2, nz+npml, nx+2*npml)``; level 1 = u^n, level 2 = u^{n-1}
* background strips: dict name -> ``(n1, n2, nt+1)`` float32, names in :data:`STRIPS`
* PML state: dicts over :data:`BP` / :data:`BU` with :func:`pml_shapes`
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))

STRIPS = ("uxl_reg", "uzl_reg", "uxr_reg", "uzr_reg", "uxb_reg", "uzb_reg",
          "uxl_pml", "uzl_pml", "uxr_pml", "uzr_pml", "uxb_pml", "uzb_pml")
BP = ("bpxlx", "bpzlx", "bpxrx", "bpzrx", "bpxtx", "bpxtz", "bpztx", "bpztz",
      "bpxbx", "bpxbz", "bpzbx", "bpzbz")
BU = tuple(f"bu{c}{k}{s}" for s in "lrbt" for c in "xz" for k in "123")

STATUS = {0: "ok", -1: "invalid argument", -2: "unsupported", -3: "out of memory", -4: "CUDA error",
          -5: "call out of order"}


class FDFKError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fdfk_gb300: {STATUS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    """fdfk_params: scalar arguments of updatedispl_ (src/FDFK2D.f90:516-519)."""
    _fields_ = [("norder", C.c_int), ("nx", C.c_int), ("nz", C.c_int), ("npml", C.c_int),
                ("is_PML_top", C.c_int), ("npower", C.c_int), ("nbd", C.c_int), ("nt", C.c_int),
                ("dx", C.c_float), ("dz", C.c_float), ("dt", C.c_double), ("vpml", C.c_float),
                ("R0", C.c_double)]

    @classmethod
    def from_dict(cls, p: dict) -> "Params":
        return cls(int(p["norder"]), int(p["nx"]), int(p["nz"]), int(p["npml"]), int(bool(p.get("is_PML_top", False))),
                   int(p.get("npower", 2)), int(p.get("nbd", 2 * int(p["norder"]) - 1)), int(p["nt"]),
                   float(p["dx"]), float(p["dz"]), float(p["dt"]), float(p["vpml"]), float(p.get("R0", 1e-3)))


class FkParams(C.Structure):
    """fdfk_fk_params: scalar arguments of comput_background_wavefield_ (src/FDFK2D.f90:429-431)."""
    _fields_ = [("nx", C.c_int), ("nz", C.c_int), ("npml", C.c_int), ("izt", C.c_int), ("nbd", C.c_int),
                ("nt", C.c_int), ("src_type", C.c_int), ("x0", C.c_float), ("z0", C.c_float), ("dx", C.c_float),
                ("dz", C.c_float), ("dt", C.c_double), ("ds", C.c_float), ("f0", C.c_float), ("rayp", C.c_double)]

    @classmethod
    def from_dict(cls, p: dict) -> "FkParams":
        return cls(int(p["nx"]), int(p["nz"]), int(p["npml"]), int(p.get("izt", 1)), int(p["nbd"]), int(p["nt"]),
                   1 if p.get("src_type", True) else 0, float(p.get("x0", 0.0)), float(p.get("z0", 0.0)),
                   float(p["dx"]), float(p["dz"]), float(p["dt"]), float(p["ds"]), float(p["f0"]),
                   float(p["rayp"]))


class SolveRequest(C.Structure):
    """fdfk_solve_request: one solve for the serving loop."""
    _fields_ = [("p", Params), ("c", C.c_void_p), ("fk", FkParams), ("bazs", C.c_void_p),
                ("nlayer_left", C.c_int), ("fk_left", C.c_void_p), ("nlayer_right", C.c_int),
                ("fk_right", C.c_void_p), ("nrcv", C.c_int), ("rx", C.c_void_p), ("rz", C.c_void_p),
                ("x0", C.c_float), ("z0", C.c_float), ("nstp", C.c_int), ("nsis", C.c_int),
                ("seisx", C.c_void_p), ("seisz", C.c_void_p)]


class ServerStats(C.Structure):
    _fields_ = [("queued", C.c_int), ("running", C.c_int), ("completed", C.c_longlong), ("failed", C.c_longlong),
                ("bytes_in_use", C.c_longlong), ("budget", C.c_longlong)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


def _fk_model(m, name):
    m = np.asfortranarray(m, np.float32)
    if m.ndim != 2 or m.shape[0] != 4:
        raise ValueError(f"{name} must have shape (4, nlayer): z_top, vp, vs, rho")
    return m


def lib_path() -> str:
    return os.path.join(PKG, "_build", "libfdfk_gb300.so")


_lib = None


def lib():
    """Load the CUDA library (fails loudly if it was not built)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise ImportError(f"fdfk_gb300 CUDA library not built: {path} (run __graft_entry__.build())")
        L = C.CDLL(path)
        L.fdfk_last_error.restype = C.c_char_p
        L.fdfk_kernel_launches.restype = C.c_longlong
        L.fdfk_session_create.argtypes = [C.POINTER(Params), C.c_void_p, C.POINTER(C.c_void_p)]
        L.fdfk_batch_destroy.restype = None
        L.fdfk_server_destroy.restype = None
        L.fdfk_input_free.restype = None
        L.fdfk_session_device_bytes.restype = C.c_longlong
        for name in ("fdfk_session_set_stream", "fdfk_session_advance", "fdfk_session_synchronize",
                     "fdfk_session_step_index", "fdfk_session_destroy", "fdfk_session_upload_background",
                     "fdfk_session_set_receivers", "fdfk_session_download_seismograms",
                     "fdfk_session_upload_state", "fdfk_session_download_state",
                     "fdfk_session_download_seismogram_range", "fdfk_session_advance_timed",
                     "fdfk_session_interior_cells", "fdfk_session_fk_background", "fdfk_fk_background",
                     "fdfk_batch_create", "fdfk_batch_add", "fdfk_batch_remove", "fdfk_batch_set_graph_chunk",
                     "fdfk_batch_set_tuning",
                     "fdfk_batch_advance", "fdfk_batch_synchronize", "fdfk_batch_live", "fdfk_batch_size",
                     "fdfk_server_create", "fdfk_server_submit", "fdfk_server_pump", "fdfk_server_request",
                     "fdfk_server_get_stats", "fdfk_input_read", "fdfk_backazimuths", "fdfk_stable_dt",
                     "fdfk_write_su", "fdfk_run", "fdfk_session_snapshot", "fdfk_session_set_tuning",
                     "fdfk_session_get_tuning", "fdfk_autotune", "fdfk_rf_itdecon"):
            getattr(L, name).restype = C.c_int if name != "fdfk_session_destroy" else None
        _lib = L
    return _lib


def kernel_launches() -> int:
    return int(lib().fdfk_kernel_launches())


def _check(rc: int):
    if rc != 0:
        raise FDFKError(rc, lib().fdfk_last_error().decode())


def _f32(a, name):
    if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.f_contiguous):
        raise TypeError(f"{name} must be a Fortran-ordered float32 array")
    return a.ctypes.data_as(C.c_void_p)


def strip_shapes(nx, nz, nbd, nt):
    """Background-strip shapes, src/FDFK2D.f90:328-355 (last axis = time 0..nt)."""
    T = nt + 1
    return {"uxl_reg": (nz - nbd, nbd, T), "uzl_reg": (nz - nbd, nbd, T),
            "uxr_reg": (nz - nbd, nbd, T), "uzr_reg": (nz - nbd, nbd, T),
            "uxb_reg": (nbd, nx, T), "uzb_reg": (nbd, nx, T),
            "uxl_pml": (nz, nbd, T), "uzl_pml": (nz, nbd, T),
            "uxr_pml": (nz, nbd, T), "uzr_pml": (nz, nbd, T),
            "uxb_pml": (nbd, nx + 2 * nbd, T), "uzb_pml": (nbd, nx + 2 * nbd, T)}


def pml_shapes(nx, nz, npml):
    """PML auxiliary-array shapes, src/FDFK2D.f90:260-306."""
    X = nx + 2 * npml
    s = {"bpxlx": (nz, npml), "bpzlx": (nz, npml), "bpxrx": (nz, npml), "bpzrx": (nz, npml)}
    for k in ("bpxtx", "bpxtz", "bpztx", "bpztz", "bpxbx", "bpxbz", "bpzbx", "bpzbz"):
        s[k] = (npml, X)
    for name in BU:
        s[name] = (2, nz, npml) if name[-1] in "lr" else (2, npml, X)
    return s


class Session:
    """Device-resident time loop of simulate_wavefield (src/FDFK2D.f90:465-532)."""

    def __init__(self, p: dict, c: np.ndarray, stream=None):
        L = lib()
        self.p = dict(p)
        self._prm = Params.from_dict(p)
        h = C.c_void_p()
        _check(L.fdfk_session_create(C.byref(self._prm), _f32(c, "c"), C.byref(h)))
        self._h = h
        self.nrcv = 0
        self.nsis = -1
        if stream is not None:
            _check(L.fdfk_session_set_stream(self._h, C.c_void_p(int(stream))))

    def close(self):
        if getattr(self, "_h", None):
            lib().fdfk_session_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload_background(self, strips: dict, t0: int = 0, count: int | None = None):
        if count is None:
            count = int(self.p["nt"]) + 1 - t0
        arr = (C.c_void_p * 12)(*[_f32(strips[k], k) for k in STRIPS])
        _check(lib().fdfk_session_upload_background(self._h, arr, C.c_int(t0), C.c_int(count)))

    def fk_background(self, p: dict, bazs, fk_left, fk_right):
        """Compute the FK background on the GPU straight into this session's strips (all times)."""
        fl, fr = _fk_model(fk_left, "fk_left"), _fk_model(fk_right, "fk_right")
        bz = np.ascontiguousarray(bazs, np.float64)
        if bz.size != int(p["nx"]) + 2 * int(p["npml"]):
            raise ValueError("bazs must hold nx + 2 npml back-azimuths")
        prm = FkParams.from_dict(p)
        _check(lib().fdfk_session_fk_background(self._h, C.byref(prm), bz.ctypes.data_as(C.c_void_p),
                                                 C.c_int(fl.shape[1]), fl.ctypes.data_as(C.c_void_p),
                                                 C.c_int(fr.shape[1]), fr.ctypes.data_as(C.c_void_p)))

    def set_receivers(self, rx, rz, x0: float, z0: float, nstp: int, nsis: int):
        rx = np.ascontiguousarray(rx, np.float32)
        rz = np.ascontiguousarray(rz, np.float32)
        _check(lib().fdfk_session_set_receivers(self._h, C.c_int(len(rx)), rx.ctypes.data_as(C.c_void_p),
                                                 rz.ctypes.data_as(C.c_void_p), C.c_float(x0), C.c_float(z0),
                                                 C.c_int(nstp), C.c_int(nsis)))
        self.nrcv, self.nsis = len(rx), nsis

    def advance(self, nsteps: int):
        _check(lib().fdfk_session_advance(self._h, C.c_int(nsteps)))

    def advance_timed(self, nsteps: int, sample_every: int = 1):
        """Advance with CUDA events around the kernels of every sample_every-th step; returns
        (ms_interior, ms_edge, ms_total): the mean time per launch of the fast-path and tiled
        kernels over the sampled steps and the time of all the steps, from one loop."""
        ti, te, tt = C.c_float(), C.c_float(), C.c_float()
        _check(lib().fdfk_session_advance_timed(self._h, C.c_int(nsteps), C.c_int(sample_every), C.byref(ti),
                                                C.byref(te), C.byref(tt)))
        return float(ti.value), float(te.value), float(tt.value)

    def cell_split(self):
        """(cells on the interior fast path, cells on the tiled kernel) per step."""
        i, e = C.c_longlong(), C.c_longlong()
        _check(lib().fdfk_session_interior_cells(self._h, C.byref(i), C.byref(e)))
        return int(i.value), int(e.value)

    @property
    def step_index(self) -> int:
        return int(lib().fdfk_session_step_index(self._h))

    def synchronize(self):
        _check(lib().fdfk_session_synchronize(self._h))

    def seismograms(self):
        sx = np.zeros((self.nsis + 1, self.nrcv), np.float32, order="F")
        sz = np.zeros_like(sx, order="F")
        _check(lib().fdfk_session_download_seismograms(self._h, _f32(sx, "seisx"), _f32(sz, "seisz")))
        return sx, sz

    def set_tuning(self, seg_len: int = 0, pml_run: int = 0):
        """Launch shapes (results do not change): fast-path segment length, absorbing-layer tile length."""
        _check(lib().fdfk_session_set_tuning(self._h, C.c_int(int(seg_len)), C.c_int(int(pml_run))))

    def tuning(self):
        a, b = C.c_int(), C.c_int()
        _check(lib().fdfk_session_get_tuning(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def snapshot(self):
        """Level 2 (u^{n-1}) of rows 1..nz, columns 1..nx as (nz, nx) arrays (ux, uz)."""
        nz, nx = int(self.p["nz"]), int(self.p["nx"])
        ux = np.zeros((nz, nx), np.float32, order="F")
        uz = np.zeros((nz, nx), np.float32, order="F")
        _check(lib().fdfk_session_snapshot(self._h, _f32(ux, "ux"), _f32(uz, "uz")))
        return ux, uz

    def seismogram_range(self, first: int, count: int, outx=None, outz=None):
        """Samples [first, first+count) of every receiver, arrays of shape (count, nrcv)."""
        sx = outx if outx is not None else np.zeros((count, self.nrcv), np.float32, order="F")
        sz = outz if outz is not None else np.zeros((count, self.nrcv), np.float32, order="F")
        _check(lib().fdfk_session_download_seismogram_range(self._h, C.c_int(first), C.c_int(count),
                                                             _f32(sx, "seisx"), _f32(sz, "seisz")))
        return sx, sz

    def upload_state(self, ux, uz, bp: dict, bu: dict, it: int):
        bpp = (C.c_void_p * 12)(*[_f32(bp[k], k) if k in bp else None for k in BP])
        bup = (C.c_void_p * 24)(*[_f32(bu[k], k) if k in bu else None for k in BU])
        _check(lib().fdfk_session_upload_state(self._h, _f32(ux, "ux"), _f32(uz, "uz"), bpp, bup, C.c_int(it)))

    def download_state(self, ux, uz, bp: dict, bu: dict):
        bpp = (C.c_void_p * 12)(*[_f32(bp[k], k) if k in bp else None for k in BP])
        bup = (C.c_void_p * 24)(*[_f32(bu[k], k) if k in bu else None for k in BU])
        _check(lib().fdfk_session_download_state(self._h, _f32(ux, "ux"), _f32(uz, "uz"), bpp, bup))


class Batch:
    """Solves (Sessions of one stencil order) advanced together: three launches per step for all
    members, chunks of steps replayed from a captured CUDA graph."""

    def __init__(self, norder: int, graph_chunk: int | None = None):
        L = lib()
        h = C.c_void_p()
        _check(L.fdfk_batch_create(C.c_int(int(norder)), C.byref(h)))
        self._h = h
        self.members = []
        if graph_chunk is not None:
            _check(L.fdfk_batch_set_graph_chunk(self._h, C.c_int(int(graph_chunk))))

    def add(self, session: "Session"):
        _check(lib().fdfk_batch_add(self._h, session._h))
        self.members.append(session)

    def set_tuning(self, seg_len: int = 0, pml_run: int = 0):
        """Launch shapes for every member while batched (0: planned for the batch / each member's
        own); the results do not depend on them."""
        _check(lib().fdfk_batch_set_tuning(self._h, C.c_int(int(seg_len)), C.c_int(int(pml_run))))

    def remove(self, session: "Session"):
        _check(lib().fdfk_batch_remove(self._h, session._h))
        self.members.remove(session)

    def advance(self, nsteps: int):
        _check(lib().fdfk_batch_advance(self._h, C.c_int(int(nsteps))))

    def synchronize(self):
        _check(lib().fdfk_batch_synchronize(self._h))

    def live(self) -> int:
        n = lib().fdfk_batch_live(self._h)
        if n < 0:
            _check(n)
        return int(n)

    def close(self):
        if getattr(self, "_h", None):
            lib().fdfk_batch_destroy(self._h)
            self._h = None
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def session_device_bytes(p: dict, nrcv: int, nsis: int) -> int:
    """Device bytes a session of these parameters holds (what the server's budget counts)."""
    prm = Params.from_dict(p)
    return int(lib().fdfk_session_device_bytes(C.byref(prm), C.c_int(nrcv), C.c_int(nsis)))


class Server:
    """Serving loop (fdfk_server): requests are admitted by device-memory budget into one running
    batch, advanced `chunk` steps per pump, and retired into host seismogram arrays when done."""

    def __init__(self, norder: int, budget_bytes: int, chunk: int = 32):
        h = C.c_void_p()
        _check(lib().fdfk_server_create(C.c_int(int(norder)), C.c_longlong(int(budget_bytes)), C.c_int(int(chunk)),
                                        C.byref(h)))
        self._h = h
        self._req = {}

    def submit(self, p: dict, c, fk: dict, bazs, fk_left, fk_right, rx, rz, x0: float = 0.0, z0: float = 0.0,
               nstp: int = 1, nsis: int | None = None) -> int:
        """Queue one solve; returns its id.  The arrays are kept alive until the request finishes."""
        if nsis is None:
            nsis = int(p["nt"]) // nstp
        keep = {"c": np.asfortranarray(c, np.float32), "bazs": np.ascontiguousarray(bazs, np.float64),
                "fl": _fk_model(fk_left, "fk_left"), "fr": _fk_model(fk_right, "fk_right"),
                "rx": np.ascontiguousarray(rx, np.float32), "rz": np.ascontiguousarray(rz, np.float32)}
        nrcv = keep["rx"].size
        keep["sx"] = np.zeros((nsis + 1, nrcv), np.float32, order="F")
        keep["sz"] = np.zeros((nsis + 1, nrcv), np.float32, order="F")
        r = SolveRequest()
        r.p = Params.from_dict(p)
        r.c = keep["c"].ctypes.data
        r.fk = FkParams.from_dict(fk)
        r.bazs = keep["bazs"].ctypes.data
        r.nlayer_left, r.fk_left = keep["fl"].shape[1], keep["fl"].ctypes.data
        r.nlayer_right, r.fk_right = keep["fr"].shape[1], keep["fr"].ctypes.data
        r.nrcv, r.rx, r.rz = nrcv, keep["rx"].ctypes.data, keep["rz"].ctypes.data
        r.x0, r.z0, r.nstp, r.nsis = float(x0), float(z0), int(nstp), int(nsis)
        r.seisx, r.seisz = keep["sx"].ctypes.data, keep["sz"].ctypes.data
        rid = C.c_longlong()
        _check(lib().fdfk_server_submit(self._h, C.byref(r), C.byref(rid)))
        self._req[rid.value] = keep
        return rid.value

    def pump(self) -> int:
        n = C.c_int()
        _check(lib().fdfk_server_pump(self._h, C.byref(n)))
        return n.value

    def request(self, rid: int):
        """(state, t_submit, t_admit, t_done) on the host steady clock (seconds)."""
        st = C.c_int()
        t = [C.c_double() for _ in range(3)]
        _check(lib().fdfk_server_request(self._h, C.c_longlong(rid), C.byref(st), *[C.byref(x) for x in t]))
        return st.value, t[0].value, t[1].value, t[2].value

    def result(self, rid: int):
        """Seismograms (seisx, seisz) of a finished request."""
        state = self.request(rid)[0]
        if state != REQ_DONE:
            raise FDFKError(-5 if state != REQ_FAILED else -1, f"request {rid} is not done (state {state})")
        keep = self._req[rid]
        return keep["sx"], keep["sz"]

    def release(self, rid: int):
        """Drop the host arrays of a finished request."""
        self._req.pop(rid, None)

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().fdfk_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().fdfk_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class InputFolder(C.Structure):
    """fdfk_input: the parsed input folder of FDFK2D (src/Input.f90)."""
    _fields_ = [("norder", C.c_int), ("nx", C.c_int), ("nz", C.c_int), ("npml", C.c_int), ("izt", C.c_int),
                ("is_PML_top", C.c_int), ("outsnap", C.c_int), ("nstep", C.c_int), ("src_type", C.c_int),
                ("nrcv", C.c_int), ("nlayer_left", C.c_int), ("nlayer_right", C.c_int),
                ("negative_velocity", C.c_int), ("x0", C.c_float), ("z0", C.c_float), ("dx", C.c_float),
                ("dz", C.c_float), ("tmax", C.c_float), ("tstp", C.c_float), ("f0", C.c_float), ("ds", C.c_float),
                ("dt", C.c_double), ("rayp", C.c_double), ("evla", C.c_double), ("evlo", C.c_double),
                ("lat_org", C.c_double), ("lon_org", C.c_double), ("az_org", C.c_double),
                ("rx", C.POINTER(C.c_float)), ("rz", C.POINTER(C.c_float)), ("fk_left", C.POINTER(C.c_float)),
                ("fk_right", C.POINTER(C.c_float)), ("c", C.POINTER(C.c_float))]


def read_input(inpath: str, inpar: str, write_model_copies: bool = False) -> dict:
    """Parse an FDFK2D input folder; returns scalars plus rx, rz, fk_left, fk_right (4, nl), c (3, NZ, NX)."""
    L = lib()
    inp = InputFolder()
    rc = L.fdfk_input_read(inpath.encode(), inpar.encode(), C.c_int(1 if write_model_copies else 0), C.byref(inp))
    try:
        _check(rc)
        out = {k: getattr(inp, k) for k, t in InputFolder._fields_ if not k in ("rx", "rz", "fk_left", "fk_right", "c")}
        NX, NZ = inp.nx + 2 * inp.npml, inp.nz + inp.npml - inp.izt + 1
        arr = lambda ptr, n: np.ctypeslib.as_array(ptr, shape=(n,)).copy()
        out["rx"] = arr(inp.rx, inp.nrcv)
        out["rz"] = arr(inp.rz, inp.nrcv)
        out["fk_left"] = np.asfortranarray(arr(inp.fk_left, 4 * inp.nlayer_left).reshape(inp.nlayer_left, 4).T)
        out["fk_right"] = np.asfortranarray(arr(inp.fk_right, 4 * inp.nlayer_right).reshape(inp.nlayer_right, 4).T)
        out["c"] = np.asfortranarray(arr(inp.c, 3 * NX * NZ).reshape(NX, NZ, 3).transpose(2, 1, 0))
        return out
    finally:
        L.fdfk_input_free(C.byref(inp))


def autotune(p: dict, c, steps: int = 20):
    """Fastest (seg_len, pml_run) for sessions of p and c, and its ms per step (fdfk_autotune)."""
    prm = Params.from_dict(p)
    a, b, ms = C.c_int(), C.c_int(), C.c_float()
    _check(lib().fdfk_autotune(C.byref(prm), _f32(c, "c"), C.c_int(int(steps)), C.byref(a), C.byref(b), C.byref(ms)))
    return a.value, b.value, ms.value


def receiver_functions(num, den, dt: float, minlag: float, maxlag: float, tshift: float = 0.0, f0: float = 8.0,
                       itmax: int = 100, minderr: float = 1e-3):
    """Receiver functions by iterative time-domain deconvolution, one per trace (fdfk_rf_itdecon; the
    computation of utils/makeRFitdecon.m, FP64 on the GPU).  num, den: (nt,) or (nt, ntr) traces, e.g. the
    radial and vertical seismograms of a solve for P-to-S.  Returns (rf (nrf, ntr), rms list of per-iteration
    misfits per trace, iterations per trace); 1-D inputs give a 1-D rf and a single rms array."""
    a = np.asarray(num, np.float32)
    b = np.asarray(den, np.float32)
    one = a.ndim == 1
    a = np.asfortranarray(a.reshape(a.shape[0], -1))
    b = np.asfortranarray(b.reshape(b.shape[0], -1))
    if a.shape != b.shape:
        raise ValueError("numerator and denominator shapes differ")
    nt, ntr = a.shape
    nrf = C.c_int()
    args = (C.c_int(nt), C.c_int(ntr), C.c_int(nt), C.c_double(dt), C.c_double(minlag), C.c_double(maxlag),
            C.c_double(tshift), C.c_double(f0), C.c_int(itmax), C.c_double(minderr))
    _check(lib().fdfk_rf_itdecon(a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), *args, None,
                                 C.c_int(0), C.byref(nrf), None, None))
    rf = np.zeros((nrf.value, ntr), np.float64, order="F")
    rms = np.zeros((max(itmax, 1), ntr), np.float64, order="F")
    its = np.zeros(ntr, np.int32)
    _check(lib().fdfk_rf_itdecon(a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), *args,
                                 rf.ctypes.data_as(C.c_void_p), C.c_int(max(nrf.value, 1)), C.byref(nrf),
                                 rms.ctypes.data_as(C.c_void_p), its.ctypes.data_as(C.c_void_p)))
    rmsl = [rms[:its[j], j].copy() for j in range(ntr)]
    if one:
        return rf[:, 0], rmsl[0], int(its[0])
    return rf, rmsl, its


def backazimuths(lat_org, lon_org, az_org, evla, evlo, coordx) -> np.ndarray:
    """Back-azimuths (rad) at profile coordinates, minus the profile azimuth (src/coord_transform.f90)."""
    x = np.ascontiguousarray(coordx, np.float32)
    out = np.zeros(x.size, np.float64)
    _check(lib().fdfk_backazimuths(C.c_double(lat_org), C.c_double(lon_org), C.c_double(az_org), C.c_double(evla),
                                   C.c_double(evlo), C.c_int(x.size), x.ctypes.data_as(C.c_void_p),
                                   out.ctypes.data_as(C.c_void_p)))
    return out


def stable_dt(norder: int, nx: int, nz: int, npml: int, dx: float, dz: float, c) -> float:
    """check_stability's stable dt (src/Submain.f90:118-164)."""
    v = C.c_double()
    _check(lib().fdfk_stable_dt(C.c_int(norder), C.c_int(nx), C.c_int(nz), C.c_int(npml), C.c_float(dx),
                                C.c_float(dz), _f32(c, "c"), C.byref(v)))
    return v.value


def write_su(path: str, data, head58: int, head59: int):
    """SU file from data (ns, ntr), one trace per column."""
    d = np.asfortranarray(data, np.float32)
    _check(lib().fdfk_write_su(path.encode(), C.c_int(d.shape[1]), C.c_int(d.shape[0]), d.ctypes.data_as(C.c_void_p),
                               C.c_int(head58), C.c_int(head59)))


def read_su(path: str, ns: int):
    """(headers (ntr, 120) int16, data (ns, ntr) float32) of an SU file of ns-sample traces."""
    raw = np.fromfile(path, np.uint8)
    rec = 240 + 4 * ns
    if raw.size % rec:
        raise ValueError(f"{path}: size is not a whole number of {ns}-sample traces")
    ntr = raw.size // rec
    r = raw.reshape(ntr, rec)
    heads = r[:, :240].copy().view(np.int16)
    data = np.asfortranarray(r[:, 240:].copy().view(np.float32).T)
    return heads, data


def run(inpath: str, inpar: str, outpath: str, fsis: str = "seis", write_model_copies: bool = True):
    """Program FDFK2D on the GPU: input folder in, <outpath>/<fsis>x.su and z.su out."""
    _check(lib().fdfk_run(inpath.encode(), inpar.encode(), outpath.encode(), fsis.encode(),
                          C.c_int(1 if write_model_copies else 0)))


def simulate(p: dict, c: np.ndarray, strips: dict, rx, rz, x0: float, z0: float, nstp: int, nsis: int):
    """The whole time loop on the GPU; returns (seisx, seisz) of shape (nsis+1, nrcv)."""
    L = lib()
    prm = Params.from_dict(p)
    rx = np.ascontiguousarray(rx, np.float32)
    rz = np.ascontiguousarray(rz, np.float32)
    sx = np.zeros((nsis + 1, len(rx)), np.float32, order="F")
    sz = np.zeros_like(sx, order="F")
    arr = (C.c_void_p * 12)(*[_f32(strips[k], k) for k in STRIPS])
    _check(L.fdfk_simulate(C.byref(prm), _f32(c, "c"), arr, C.c_int(len(rx)), rx.ctypes.data_as(C.c_void_p),
                           rz.ctypes.data_as(C.c_void_p), C.c_float(x0), C.c_float(z0), C.c_int(nstp),
                           C.c_int(nsis), _f32(sx, "seisx"), _f32(sz, "seisz")))
    return sx, sz


def fk_background(p: dict, bazs, fk_left, fk_right) -> dict:
    """comput_background_wavefield on the GPU: the 12 strips as Fortran-ordered float32 host arrays.

    p: nx, nz, npml, nbd, nt, dt, dx, dz, x0, z0, ds, f0, rayp (s/m), src_type (True = P).
    bazs: back-azimuths (rad) of the nx + 2 npml columns; fk_left / fk_right: (4, nlayer)
    z_top, vp, vs, rho per layer, the last the half-space.
    """
    fl, fr = _fk_model(fk_left, "fk_left"), _fk_model(fk_right, "fk_right")
    bz = np.ascontiguousarray(bazs, np.float64)
    if bz.size != int(p["nx"]) + 2 * int(p["npml"]):
        raise ValueError("bazs must hold nx + 2 npml back-azimuths")
    out = {k: np.zeros(sh, np.float32, order="F")
           for k, sh in strip_shapes(int(p["nx"]), int(p["nz"]), int(p["nbd"]), int(p["nt"])).items()}
    arr = (C.c_void_p * 12)(*[_f32(out[k], k) for k in STRIPS])
    prm = FkParams.from_dict(p)
    _check(lib().fdfk_fk_background(C.byref(prm), bz.ctypes.data_as(C.c_void_p), C.c_int(fl.shape[1]),
                                    fl.ctypes.data_as(C.c_void_p), C.c_int(fr.shape[1]),
                                    fr.ctypes.data_as(C.c_void_p), arr))
    return out


def comput_background_wavefield(p: dict, bazs, fk_left, fk_right, strips: dict):
    """The reference entry point comput_background_wavefield_ (32 arguments), on the GPU, in place."""
    L = lib()
    i = lambda v: C.byref(C.c_int(int(v)))
    f = lambda v: C.byref(C.c_float(float(v)))
    d = lambda v: C.byref(C.c_double(float(v)))
    fl, fr = _fk_model(fk_left, "fk_left"), _fk_model(fk_right, "fk_right")
    bz = np.ascontiguousarray(bazs, np.float64)
    args = [i(p["nx"]), i(p["nz"]), i(p["npml"]), i(p.get("izt", 1)), i(p["nbd"]), i(p["nt"]), i(fl.shape[1]),
            i(fr.shape[1]), i(1 if p.get("src_type", True) else 0), f(p.get("x0", 0.0)), f(p.get("z0", 0.0)),
            f(p["dx"]), f(p["dz"]), d(p["dt"]), f(p["ds"]), f(p["f0"]), d(p["rayp"]),
            bz.ctypes.data_as(C.c_void_p), fl.ctypes.data_as(C.c_void_p), fr.ctypes.data_as(C.c_void_p)]
    args += [_f32(strips[k], k) for k in STRIPS]
    L.comput_background_wavefield_(*args)


def updatedispl(p: dict, strips: dict, c, coef0, coef1, ux, uz, bp: dict, bu: dict, it: int):
    """The reference entry point updatedispl_ (68 arguments), executed on the GPU in place."""
    L = lib()
    i = lambda v: C.byref(C.c_int(int(v)))
    f = lambda v: C.byref(C.c_float(float(v)))
    d = lambda v: C.byref(C.c_double(float(v)))
    norder = int(p["norder"])
    izt = 1 - int(p["npml"]) if p.get("is_PML_top", False) else 1
    args = [i(norder), i(p["nx"]), i(p["nz"]), i(p["npml"]), i(izt), i(1 if p.get("is_PML_top", False) else 0),
            i(p.get("npower", 2)), i(p.get("nbd", 2 * norder - 1)), i(it), i(p["nt"]), f(p["dx"]), f(p["dz"]),
            d(p["dt"]), f(p["vpml"]), d(p.get("R0", 1e-3))]
    args += [_f32(strips[k], k) for k in STRIPS]
    c0 = np.asfortranarray(coef0, np.float64)
    c1 = np.asfortranarray(coef1, np.float64)
    args += [_f32(c, "c"), c0.ctypes.data_as(C.c_void_p), c1.ctypes.data_as(C.c_void_p), _f32(ux, "ux"), _f32(uz, "uz")]
    args += [_f32(bp[k], k) for k in BP]
    args += [_f32(bu[k], k) for k in BU]
    L.updatedispl_(*args)
