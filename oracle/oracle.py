"""TEST INFRASTRUCTURE ONLY: ctypes view of the C oracle (oracle/fem_oracle.c).

Imported by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg,
always as the parity reference / CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfem_oracle.so")

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


class _Problem(C.Structure):
    _fields_ = [("dim", C.c_int32), ("n_nodes", C.c_int64), ("n_elems", C.c_int64),
                ("nodes", C.c_void_p), ("elems", C.c_void_p), ("n_constraints", C.c_int64),
                ("cons", C.c_void_p), ("n_loads", C.c_int64), ("load_node", C.c_void_p),
                ("load_vec", C.c_void_p), ("n_faces", C.c_int64), ("face_nodes", C.c_void_p),
                ("face_elem", C.c_void_p), ("face_normal", C.c_void_p), ("face_pressure", C.c_void_p),
                ("elem_E", C.c_void_p), ("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("consistent", C.c_int32)]


class _Wavelet(C.Structure):
    _fields_ = [("type", C.c_int32), ("freq", C.c_double), ("timeshift", C.c_double), ("ampl", C.c_double)]


class _Dyn(C.Structure):
    _fields_ = [("beta1", C.c_double), ("beta2", C.c_double), ("dt", C.c_double), ("endtime", C.c_double)]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP when available)."""
    src = os.path.join(HERE, "fem_oracle.c")
    deps = [src, os.path.join(HERE, "ebe_port.inc"), os.path.join(HERE, "fem_oracle.h")]
    if not force and os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d) for d in deps):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    base = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", src, "-o", LIB_PATH, "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True, capture_output=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P, W, D = C.POINTER(_Problem), C.POINTER(_Wavelet), C.POINTER(_Dyn)
        L.orc_wavelet_value_f32.restype = C.c_float
        L.orc_wavelet_value_f32.argtypes = [W, C.c_float]
        L.orc_ebe_static_f32.argtypes = [P, W, C.c_double, _f32p, C.POINTER(C.c_int32)]
        L.orc_ebe_static_f64.argtypes = [P, W, C.c_double, _f64p, C.POINTER(C.c_int32)]
        L.orc_ebe_dyn_f32.argtypes = [P, W, D, _f32p, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
        L.orc_ebe_dyn_f64.argtypes = [P, W, D, _f64p, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
        L.orc_ebe_setup_f32.argtypes = [P, W] + [C.c_void_p] * 6
        L.orc_ebe_time_f32.argtypes = [P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_setup.argtypes = [P, C.POINTER(C.c_void_p)]
        L.orc_assemble.argtypes = [C.c_void_p]
        L.orc_pcg_warm.argtypes = [C.c_void_p, _f64p, _f64p, C.c_double, C.c_int32, C.c_int32,
                                   C.POINTER(C.c_int32)]
        L.orc_ebe_timer_create.argtypes = [P, C.POINTER(C.c_void_p)]
        L.orc_ebe_timer_iters.restype = C.c_double
        L.orc_ebe_timer_iters.argtypes = [C.c_void_p, C.c_int32]
        L.orc_ebe_timer_info.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_ebe_timer_free.argtypes = [C.c_void_p]
        L.orc_num_threads.restype = C.c_int
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_ndof.restype = C.c_int64
        L.orc_ndof.argtypes = [C.c_void_p]
        L.orc_get_mask.argtypes = [C.c_void_p, _i32p]
        L.orc_get_adjacency.argtypes = [C.c_void_p, _i32p]
        L.orc_get_bc.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")]
        L.orc_get_element_matrices.argtypes = [C.c_void_p, _f64p]
        L.orc_get_diag.argtypes = [C.c_void_p, _f64p]
        L.orc_get_rhs.argtypes = [C.c_void_p, W, C.c_double, _f64p]
        L.orc_matvec.argtypes = [C.c_void_p, _f64p, _f64p]
        L.orc_pcg.argtypes = [C.c_void_p, _f64p, _f64p, C.c_double, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]
        L.orc_dyn_run.argtypes = [C.c_void_p, W, D, C.c_double, C.c_int32, _f64p, C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int64)]
        L.orc_grad_E.argtypes = [C.c_void_p, _f64p, _f64p, _f64p]
        L.orc_element_stress.argtypes = [C.c_void_p, _f64p, _f64p, _f64p, _f64p]
        L.orc_dyn_adjoint.restype = C.c_double
        L.orc_dyn_adjoint.argtypes = [C.c_void_p, W, D, C.c_int32, _i32p, _f64p, _f64p]
        _lib = L
    return _lib


class _Packed:
    """Keeps numpy arrays alive while the C struct points at them."""

    def __init__(self, p, consistent: bool):
        c = lambda a, dt: np.ascontiguousarray(a, dtype=dt)
        self.nodes = c(p.nodes, np.float64)
        self.elems = c(p.elems, np.int32)
        self.cons = c(p.cons.reshape(-1, 2), np.int32)
        self.lnode = c(p.load_node, np.int32)
        self.lvec = c(p.load_vec.reshape(-1, p.dim) if len(p.load_node) else np.zeros((0, p.dim)), np.float64)
        self.fnodes = c(p.face_nodes.reshape(-1, p.dim + 1), np.int32)
        self.felem = c(p.face_elem, np.int32)
        self.fnorm = c(p.face_normal.reshape(-1, p.dim) if len(p.face_elem) else np.zeros((0, p.dim)), np.float64)
        self.fpress = c(p.face_pressure, np.float64)
        self.elemE = None if p.elem_E is None else c(p.elem_E, np.float64)
        ptr = lambda a: a.ctypes.data if a is not None and a.size else None
        self.s = _Problem(p.dim, p.n_nodes, p.n_elems, ptr(self.nodes), ptr(self.elems), len(self.cons),
                          ptr(self.cons), len(self.lnode), ptr(self.lnode), ptr(self.lvec), len(self.felem),
                          ptr(self.fnodes), ptr(self.felem), ptr(self.fnorm), ptr(self.fpress),
                          ptr(self.elemE), float(p.E), float(p.nu), float(p.rho), int(consistent))


def wavelet_struct(w=None) -> _Wavelet:
    if w is None:
        return _Wavelet(0, 15.0, 0.0, 1.0)
    return _Wavelet(int(w.code), float(w.freq), float(w.timeshift), float(w.ampl))


def wavelet_value(w, t: float) -> float:
    ws = wavelet_struct(w)
    return float(lib().orc_wavelet_value_f32(C.byref(ws), C.c_float(t)))


def ebe_static(p, wavelet=None, eps=1e-8, f64=False):
    """Element-local restatement of gpuCalculateFEM_EbE_vec; returns (u [N,dim], iterations)."""
    pk = _Packed(p, False)
    out = np.zeros(p.n_dof, np.float64 if f64 else np.float32)
    it = C.c_int32(0)
    fn = lib().orc_ebe_static_f64 if f64 else lib().orc_ebe_static_f32
    rc = fn(C.byref(pk.s), C.byref(wavelet_struct(wavelet)), float(eps), out, C.byref(it))
    if rc:
        raise RuntimeError(f"oracle ebe_static failed: {rc}")
    return out.reshape(-1, p.dim), it.value


def ebe_dyn(p, beta1, beta2, dt, endtime, wavelet=None, f64=False):
    pk = _Packed(p, False)
    out = np.zeros(p.n_dof, np.float64 if f64 else np.float32)
    st, it = C.c_int32(0), C.c_int64(0)
    fn = lib().orc_ebe_dyn_f64 if f64 else lib().orc_ebe_dyn_f32
    d = _Dyn(beta1, beta2, dt, endtime)
    rc = fn(C.byref(pk.s), C.byref(wavelet_struct(wavelet)), C.byref(d), out, C.byref(st), C.byref(it))
    if rc:
        raise RuntimeError(f"oracle ebe_dyn failed: {rc}")
    return out.reshape(-1, p.dim), st.value, it.value


def ebe_setup(p, wavelet=None):
    """Setup arrays in the reference's float layout: mask, adj, Klocals, diagK, Flocals, areas."""
    pk = _Packed(p, False)
    w = 6 * (p.dim - 1)
    out = dict(mask=np.zeros(p.n_elems * w, np.float32), adj=np.zeros(p.n_dof, np.float32),
               Klocals=np.zeros(p.n_elems * w * w, np.float32), diagK=np.zeros(p.n_elems * w, np.float32),
               Flocals=np.zeros(p.n_elems * w, np.float32), areas=np.zeros(p.n_elems, np.float32))
    rc = lib().orc_ebe_setup_f32(C.byref(pk.s), C.byref(wavelet_struct(wavelet)),
                                 *[out[k].ctypes.data for k in ("mask", "adj", "Klocals", "diagK", "Flocals", "areas")])
    if rc:
        raise RuntimeError(f"oracle ebe_setup failed: {rc}")
    return out


def ebe_time(p, k):
    pk = _Packed(p, False)
    s, i = C.c_double(0), C.c_double(0)
    rc = lib().orc_ebe_time_f32(C.byref(pk.s), int(k), C.byref(s), C.byref(i))
    if rc:
        raise RuntimeError(f"oracle ebe_time failed: {rc}")
    return s.value, i.value


def num_threads() -> int:
    return int(lib().orc_num_threads())


class EbeTimer:
    """The FP32 port of the reference's PCG, set up once and timed in samples
    of k iterations (the reference arm of the benchmark)."""

    def __init__(self, p):
        self._pk = _Packed(p, False)
        self._h = C.c_void_p()
        rc = lib().orc_ebe_timer_create(C.byref(self._pk.s), C.byref(self._h))
        if rc:
            raise RuntimeError(f"oracle timer setup failed: {rc}")
        s, i = C.c_double(0), C.c_double(0)
        lib().orc_ebe_timer_info(self._h, C.byref(s), C.byref(i))
        self.setup_s, self.init_s = s.value, i.value

    def iters(self, k: int) -> float:
        """Wall seconds of k more PCG iterations."""
        return float(lib().orc_ebe_timer_iters(self._h, int(k)))

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_ebe_timer_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Oracle:
    """FP64 global-vector oracle (compat or consistent)."""

    def __init__(self, p, consistent: bool = False):
        self.p = p
        self._pk = _Packed(p, consistent)
        self._h = C.c_void_p()
        rc = lib().orc_setup(C.byref(self._pk.s), C.byref(self._h))
        if rc:
            raise RuntimeError(f"oracle setup failed: {rc}")
        self.ndof = int(lib().orc_ndof(self._h))
        self.w = 6 * (p.dim - 1)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_free(self._h)
            self._h = None

    def assemble(self):
        """Switch matvecs and solves to the assembled node-block copy of K'
        (same element matrices, other summation order: large meshes)."""
        rc = lib().orc_assemble(self._h)
        if rc:
            raise RuntimeError(f"oracle assemble failed: {rc}")
        return self

    def mask(self):
        m = np.zeros(self.p.n_elems * self.w, np.int32)
        lib().orc_get_mask(self._h, m)
        return m

    def adjacency(self):
        a = np.zeros(self.ndof, np.int32)
        lib().orc_get_adjacency(self._h, a)
        return a

    def bc(self):
        b = np.zeros(self.ndof, np.uint8)
        lib().orc_get_bc(self._h, b)
        return b

    def element_matrices(self):
        k = np.zeros(self.p.n_elems * self.w * self.w, np.float64)
        lib().orc_get_element_matrices(self._h, k)
        return k.reshape(-1, self.w, self.w)

    def diag(self):
        d = np.zeros(self.ndof, np.float64)
        lib().orc_get_diag(self._h, d)
        return d

    def rhs(self, wavelet=None, t=0.0):
        f = np.zeros(self.ndof, np.float64)
        lib().orc_get_rhs(self._h, C.byref(wavelet_struct(wavelet)), float(t), f)
        return f

    def matvec(self, x):
        y = np.zeros(self.ndof, np.float64)
        lib().orc_matvec(self._h, np.ascontiguousarray(x, np.float64), y)
        return y

    def pcg(self, f, tol=1e-12, rule=1, maxit=1000000, allow_maxit=False):
        x = np.zeros(self.ndof, np.float64)
        it = C.c_int32(0)
        rc = lib().orc_pcg(self._h, np.ascontiguousarray(f, np.float64), x, float(tol), int(rule), int(maxit),
                           C.byref(it))
        if rc not in ((0, -4) if allow_maxit else (0,)):
            raise RuntimeError(f"oracle pcg failed: {rc}")
        return x, it.value

    def pcg_warm(self, f, x0, tol=1e-12, rule=1, maxit=1000000):
        """Jacobi PCG from the iterate x0 (returns a new array)."""
        x = np.array(x0, dtype=np.float64, copy=True)
        it = C.c_int32(0)
        rc = lib().orc_pcg_warm(self._h, np.ascontiguousarray(f, np.float64), x, float(tol), int(rule), int(maxit),
                                C.byref(it))
        if rc:
            raise RuntimeError(f"oracle pcg failed: {rc}")
        return x, it.value

    def static(self, tol=1e-12, rule=1, wavelet=None):
        return self.pcg(self.rhs(wavelet, 0.0), tol=tol, rule=rule)

    def dyn(self, beta1, beta2, dt, endtime, wavelet=None, pcg_tol=1e-12, pcg_rule=1):
        u = np.zeros(self.ndof, np.float64)
        st, it = C.c_int32(0), C.c_int64(0)
        d = _Dyn(beta1, beta2, dt, endtime)
        rc = lib().orc_dyn_run(self._h, C.byref(wavelet_struct(wavelet)), C.byref(d), float(pcg_tol), int(pcg_rule),
                               u, C.byref(st), C.byref(it))
        if rc:
            raise RuntimeError(f"oracle dyn failed: {rc}")
        return u, st.value, it.value

    def dyn_adjoint(self, beta1, dt, endtime, rec_nodes, obs, wavelet=None):
        """Explicit GN22 receiver-misfit loss and dL/dE per element (discrete adjoint)."""
        rec = np.ascontiguousarray(rec_nodes, np.int32)
        g = np.zeros(self.p.n_elems, np.float64)
        d = _Dyn(beta1, 0.0, dt, endtime)
        L = lib().orc_dyn_adjoint(self._h, C.byref(wavelet_struct(wavelet)), C.byref(d), len(rec), rec,
                                  np.ascontiguousarray(obs, np.float64).ravel(), g)
        return L, g

    def element_stress(self, u):
        """(strain, stress, von Mises) per element of displacements u."""
        s = 3 * (self.p.dim - 1)
        eps = np.zeros(self.p.n_elems * s)
        sig = np.zeros(self.p.n_elems * s)
        mis = np.zeros(self.p.n_elems)
        lib().orc_element_stress(self._h, np.ascontiguousarray(u, np.float64).ravel(), eps, sig, mis)
        return eps.reshape(-1, s), sig.reshape(-1, s), mis

    def grad_E(self, lam, u):
        g = np.zeros(self.p.n_elems, np.float64)
        lib().orc_grad_E(self._h, np.ascontiguousarray(lam, np.float64), np.ascontiguousarray(u, np.float64), g)
        return g
