"""Python driver over the C-ABI (include/cfem.h).

:class:`FemContext` mirrors the reference's pair ``dataKeeper`` +
``ElementsData::setElementsData`` (datakeeper.cpp:246-252, fem_utils.cpp:41-51)
and offers its solver entry points:

* :meth:`FemContext.static_solve`  -> gpuCalculateFEM_EbE_vec (femfunc.cpp:3-23)
* :meth:`FemContext.pcg`           -> gpuPCG_EbE_vec (femfunc.cpp:25-128)
* :meth:`FemContext.dyn`           -> gpuCalculateFEM_DYN (femfunc.cpp:130-381)

Arrays may be numpy (host) or CUDA torch tensors (device pointers are passed
straight through; no host round trip).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import capi
from .meshio import Problem, WaveletParams

_PREC = {"fp64": capi.FP64, "fp32": capi.FP32, "fp32_refine": capi.FP32_REFINE, "refine": capi.FP32_REFINE}
_RULE = {"reference": capi.STOP_REFERENCE, "residual": capi.STOP_RESIDUAL}


def _ptr(a):
    """Pointer of a numpy array or a torch tensor (device or host)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def _wavelet(w: Optional[WaveletParams]):
    if w is None:
        return None
    return capi.Wavelet(int(w.code), float(w.freq), float(w.timeshift), float(w.ampl))


def _mesh_struct(p: Problem):
    """cfem_mesh view of a Problem; the returned dict keeps its arrays alive."""
    c = lambda a, dt: np.ascontiguousarray(a, dtype=dt)
    k = dict(
        nodes=c(p.nodes, np.float64), elems=c(p.elems, np.int32), cons=c(p.cons.reshape(-1, 2), np.int32),
        lnode=c(p.load_node, np.int32), lvec=c(p.load_vec.reshape(-1, p.dim) if len(p.load_node) else np.zeros((0, p.dim)), np.float64),
        fnodes=c(p.face_nodes.reshape(-1, p.dim + 1), np.int32), felem=c(p.face_elem, np.int32),
        fnorm=c(p.face_normal.reshape(-1, p.dim) if len(p.face_elem) else np.zeros((0, p.dim)), np.float64),
        fpress=c(p.face_pressure, np.float64),
        young=None if p.elem_E is None else c(p.elem_E, np.float64))
    pz = lambda a: a.ctypes.data if a is not None and a.size else None
    mesh = capi.Mesh(p.dim, p.n_nodes, pz(k["nodes"]), p.n_elems, pz(k["elems"]), len(k["cons"]), pz(k["cons"]),
                     len(k["lnode"]), pz(k["lnode"]), pz(k["lvec"]), len(k["felem"]), pz(k["fnodes"]),
                     pz(k["felem"]), pz(k["fnorm"]), pz(k["fpress"]), pz(k["young"]))
    return mesh, k


def autotune_patch_elems(p: Problem, semantics: str = "compat", matvec_form: str = "auto", candidates=None):
    """Elements per CTA patch for this mesh on the current GPU
    (cfem_autotune_patch_elems): returns (best, {candidate: ms per matvec})."""
    mesh, keep = _mesh_struct(p)
    mat = capi.Material(float(p.E), float(p.nu), float(p.rho))
    form = {"gradient": capi.FORM_GRADIENT, "auto": capi.FORM_AUTO, "fan": capi.FORM_GRADIENT_FAN,
            "geometry": capi.FORM_GEOMETRY_FAN}[matvec_form]
    opt = capi.Options({"compat": capi.COMPAT, "consistent": capi.CONSISTENT}[semantics], form, 0, 0)
    cand = None if candidates is None else np.ascontiguousarray(candidates, np.int32)
    n = 0 if cand is None else len(cand)
    times = np.zeros(max(n, 4 if p.dim == 3 and matvec_form != "gradient" else 3))
    best = C.c_int32(0)
    st = capi.lib().cfem_autotune_patch_elems(C.byref(mesh), C.byref(mat), C.byref(opt),
                                              None if cand is None else cand.ctypes.data, n, C.byref(best),
                                              times.ctypes.data)
    capi.check(st, "cfem_autotune_patch_elems")
    used = list(cand) if cand is not None else ([192, 384, 576, 768] if p.dim == 3 and matvec_form != "gradient"
                                                  else [256, 512, 1024])
    return int(best.value), dict(zip(used, times[:len(used)].tolist()))


class FemContext:
    """One mesh on the current GPU. ``semantics`` is "compat" (reproduce the
    reference, quirks included) or "consistent" (textbook operators/loads)."""

    def __init__(self, p: Problem, semantics: str = "compat", stream=None, patch_elems: int = 0,
                 verbose: bool = False, matvec_form: str = "auto"):
        self.p = p
        self.dim = p.dim
        self.n_nodes = p.n_nodes
        self.n_elems = p.n_elems
        self.ndof = p.n_dof
        self.w = 6 * (p.dim - 1)
        L = capi.lib()
        if patch_elems == "auto":
            patch_elems, _ = autotune_patch_elems(p, semantics, matvec_form)
        self.patch_elems = int(patch_elems)
        mesh, self._keep = _mesh_struct(p)
        mat = capi.Material(float(p.E), float(p.nu), float(p.rho))
        form = {"gradient": capi.FORM_GRADIENT, "stored_ke": capi.FORM_STORED_KE, "auto": capi.FORM_AUTO,
                "fan": capi.FORM_GRADIENT_FAN, "geometry": capi.FORM_GEOMETRY_FAN}[matvec_form]
        opt = capi.Options({"compat": capi.COMPAT, "consistent": capi.CONSISTENT}[semantics], form, int(patch_elems),
                           int(verbose))
        h = C.c_void_p()
        st = L.cfem_create(C.byref(h), C.byref(mesh), C.byref(mat), C.byref(opt), stream)
        capi.check(st, "cfem_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().cfem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------- setup products
    def counts(self):
        out = np.zeros(6, np.int64)
        capi.check(capi.lib().cfem_get_counts(self._h, out.ctypes.data), "cfem_get_counts")
        return dict(zip(["dim", "n_nodes", "n_elems", "n_dof", "n_patches", "matvec_form"], out.tolist()))

    def dof_map(self):
        m = np.zeros(self.n_elems * self.w, np.int32)
        capi.check(capi.lib().cfem_dof_map(self._h, m.ctypes.data), "cfem_dof_map")
        return m

    def adjacency(self):
        a = np.zeros(self.ndof, np.int32)
        capi.check(capi.lib().cfem_adjacency(self._h, a.ctypes.data), "cfem_adjacency")
        return a

    def bc_mask(self):
        b = np.zeros(self.ndof, np.uint8)
        capi.check(capi.lib().cfem_bc_mask(self._h, b.ctypes.data), "cfem_bc_mask")
        return b

    def renumbering(self):
        n = np.zeros(self.n_nodes, np.int32)
        e = np.zeros(self.n_elems, np.int32)
        capi.check(capi.lib().cfem_renumbering(self._h, n.ctypes.data, e.ctypes.data), "cfem_renumbering")
        return n, e

    def element_matrices(self, first=0, count=None):
        count = self.n_elems - first if count is None else count
        k = np.zeros(count * self.w * self.w, np.float64)
        capi.check(capi.lib().cfem_element_matrices(self._h, first, count, k.ctypes.data), "cfem_element_matrices")
        return k.reshape(count, self.w, self.w)

    def diagonal(self):
        d = np.zeros(self.ndof, np.float64)
        capi.check(capi.lib().cfem_diagonal(self._h, d.ctypes.data), "cfem_diagonal")
        return d

    def rhs(self, wavelet: Optional[WaveletParams] = None, t: float = 0.0):
        f = np.zeros(self.ndof, np.float64)
        w = _wavelet(wavelet)
        capi.check(capi.lib().cfem_rhs(self._h, C.byref(w) if w else None, float(t), f.ctypes.data), "cfem_rhs")
        return f

    # ---------------------------------------------------------- operators / solvers
    def matvec(self, x, precision: str = "fp64", out=None):
        dt = np.float64 if precision == "fp64" else np.float32
        if out is None:
            if hasattr(x, "data_ptr"):
                import torch
                out = torch.empty_like(x)
            else:
                out = np.zeros(self.ndof, dt)
                x = np.ascontiguousarray(x, dtype=dt)
        capi.check(capi.lib().cfem_matvec(self._h, _PREC[precision], _ptr(x), _ptr(out)), "cfem_matvec")
        return out

    @staticmethod
    def _params(precision, tol, stop_rule, max_iter, outer_tol, max_outer):
        return capi.SolveParams(_PREC[precision], _RULE[stop_rule], float(tol), int(max_iter), float(outer_tol),
                                int(max_outer))

    @staticmethod
    def _info(inf):
        return dict(status=inf.status, iterations=inf.iterations, outer_iterations=inf.outer_iterations,
                    rel_residual=inf.rel_residual, gamma0=inf.gamma0, gamma=inf.gamma, solve_ms=inf.solve_ms,
                    kernel_launches=inf.kernel_launches)

    def static_solve(self, precision="fp64", tol=1e-8, stop_rule="reference", max_iter=1000000, outer_tol=1e-12,
                     max_outer=50, wavelet: Optional[WaveletParams] = None, out=None, allow_not_converged=False):
        """gpuCalculateFEM_EbE_vec: returns (u [n_nodes, dim] float64, info)."""
        u = np.zeros(self.ndof, np.float64) if out is None else out
        prm = self._params(precision, tol, stop_rule, max_iter, outer_tol, max_outer)
        inf = capi.SolveInfo()
        w = _wavelet(wavelet)
        st = capi.lib().cfem_static_solve(self._h, C.byref(w) if w else None, C.byref(prm), _ptr(u), C.byref(inf))
        capi.check(st, "cfem_static_solve", (capi.OK, capi.ERR_NOT_CONVERGED) if allow_not_converged else (capi.OK,))
        return (u.reshape(-1, self.dim) if out is None else u), self._info(inf)

    def pcg(self, f, precision="fp64", tol=1e-8, stop_rule="reference", max_iter=1000000, outer_tol=1e-12,
            max_outer=50, out=None, allow_not_converged=False):
        """gpuPCG_EbE_vec for an explicit right-hand side f (caller order, n_dof)."""
        if out is None:
            if hasattr(f, "data_ptr"):
                import torch
                out = torch.zeros_like(f)
            else:
                out = np.zeros(self.ndof, np.float64)
                f = np.ascontiguousarray(f, dtype=np.float64)
        prm = self._params(precision, tol, stop_rule, max_iter, outer_tol, max_outer)
        inf = capi.SolveInfo()
        st = capi.lib().cfem_pcg(self._h, C.byref(prm), _ptr(f), _ptr(out), C.byref(inf))
        capi.check(st, "cfem_pcg", (capi.OK, capi.ERR_NOT_CONVERGED) if allow_not_converged else (capi.OK,))
        return out, self._info(inf)

    def pcg_multi(self, F, precision="fp64", tol=1e-8, stop_rule="reference", max_iter=1000000, outer_tol=1e-12,
                  max_outer=50, allow_not_converged=False):
        """k load cases at once: F [k][n_dof] -> U [k][n_dof], per-case infos."""
        F = np.ascontiguousarray(F, dtype=np.float64)
        k = F.shape[0]
        U = np.zeros_like(F)
        prm = self._params(precision, tol, stop_rule, max_iter, outer_tol, max_outer)
        infos = (capi.SolveInfo * k)()
        st = capi.lib().cfem_pcg_multi(self._h, C.byref(prm), k, F.ctypes.data, U.ctypes.data, infos)
        capi.check(st, "cfem_pcg_multi", (capi.OK, capi.ERR_NOT_CONVERGED) if allow_not_converged else (capi.OK,))
        return U, [self._info(i) for i in infos]

    def adjoint(self, u, dLdu, precision="fp64", tol=1e-12, stop_rule="residual", max_iter=1000000, outer_tol=1e-13,
                max_outer=50):
        """lambda = K'^-1 dL/du; returns (dL/dE per element, dL/df = lambda, info).
        With CUDA float64 tensors for u and dL/du the outputs are CUDA tensors
        and nothing passes through the host."""
        if hasattr(u, "data_ptr") and hasattr(dLdu, "data_ptr"):
            import torch
            u = u.contiguous().view(-1)
            g = dLdu.contiguous().view(-1)
            dE = torch.empty(self.n_elems, dtype=torch.float64, device=u.device)
            df = torch.empty(self.ndof, dtype=torch.float64, device=u.device)
        else:
            u = np.ascontiguousarray(u, dtype=np.float64).ravel()
            g = np.ascontiguousarray(dLdu, dtype=np.float64).ravel()
            dE = np.zeros(self.n_elems, np.float64)
            df = np.zeros(self.ndof, np.float64)
        prm = self._params(precision, tol, stop_rule, max_iter, outer_tol, max_outer)
        inf = capi.SolveInfo()
        st = capi.lib().cfem_adjoint(self._h, C.byref(prm), _ptr(u), _ptr(g), _ptr(dE), _ptr(df), C.byref(inf))
        capi.check(st, "cfem_adjoint")
        return dE, df, self._info(inf)

    def element_stress(self, u):
        """Per-element (strain, stress, von Mises) of displacements u (caller order)."""
        s = 3 * (self.dim - 1)
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        eps = np.zeros((self.n_elems, s))
        sig = np.zeros((self.n_elems, s))
        mis = np.zeros(self.n_elems)
        capi.check(capi.lib().cfem_element_stress(self._h, u.ctypes.data, eps.ctypes.data, sig.ctypes.data,
                                                  mis.ctypes.data), "cfem_element_stress")
        return eps, sig, mis

    def dyn_adjoint(self, beta1, dt, endtime, receivers, obs, wavelet: Optional[WaveletParams] = None):
        """Explicit GN22 receiver-misfit loss and dL/dE (sqrt(N)-checkpointed adjoint)."""
        rec = np.ascontiguousarray(receivers, dtype=np.int32)
        obs = np.ascontiguousarray(obs, dtype=np.float64)
        g = np.zeros(self.n_elems)
        L = C.c_double(0)
        prm = capi.DynParams(float(beta1), 0.0, float(dt), float(endtime), capi.FP64, 0.0, 0, 0, 0, 0, None, None)
        inf = capi.DynInfo()
        w = _wavelet(wavelet)
        capi.check(capi.lib().cfem_dyn_adjoint(self._h, C.byref(prm), C.byref(w) if w else None, len(rec),
                                               rec.ctypes.data, obs.ctypes.data, C.byref(L), g.ctypes.data,
                                               C.byref(inf)), "cfem_dyn_adjoint")
        return L.value, g, dict(steps=inf.steps, solve_ms=inf.solve_ms)

    def set_young(self, young):
        """Per-element Young's moduli [n_elems]: numpy, or a CUDA float64 tensor (read on the device)."""
        y = young.contiguous() if hasattr(young, "data_ptr") else np.ascontiguousarray(young, dtype=np.float64)
        capi.check(capi.lib().cfem_set_young(self._h, _ptr(y)), "cfem_set_young")

    def set_stream(self, stream):
        """Issue this context's work on ``stream`` (a cudaStream_t as an int, or
        a torch.cuda.Stream); 0 / None: the legacy default stream, followed by a
        stream of the context's own. Captured graphs are dropped on a change."""
        s = getattr(stream, "cuda_stream", stream) or 0
        if getattr(self, "_stream", 0) == s:
            return
        capi.check(capi.lib().cfem_set_stream(self._h, C.c_void_p(s) if s else None), "cfem_set_stream")
        self._stream = s

    def dyn(self, beta1, beta2, dt, endtime, precision="fp64", wavelet: Optional[WaveletParams] = None,
            pcg_tol=1e-10, stop_rule="residual", max_iter=1000000, warm_start=True, receivers=None):
        """gpuCalculateFEM_DYN: returns (u [n_nodes, dim], info[, trace])."""
        u = np.zeros(self.ndof, np.float64)
        rec = None if receivers is None else np.ascontiguousarray(receivers, dtype=np.int32)
        nsteps = 1 if np.float32(endtime) < 0 else max(1, int(np.float32(endtime) / np.float32(dt)))
        trace = None if rec is None else np.zeros((nsteps, len(rec), self.dim), np.float64)
        prm = capi.DynParams(float(beta1), float(beta2), float(dt), float(endtime), _PREC[precision], float(pcg_tol),
                             _RULE[stop_rule], int(max_iter), int(warm_start), 0 if rec is None else len(rec),
                             None if rec is None else rec.ctypes.data, None if trace is None else trace.ctypes.data)
        inf = capi.DynInfo()
        w = _wavelet(wavelet)
        st = capi.lib().cfem_dyn(self._h, C.byref(prm), C.byref(w) if w else None, u.ctypes.data, C.byref(inf))
        capi.check(st, "cfem_dyn")
        info = dict(status=inf.status, steps=inf.steps, pcg_iterations=inf.pcg_iterations, solve_ms=inf.solve_ms)
        if trace is not None:
            return u.reshape(-1, self.dim), info, trace
        return u.reshape(-1, self.dim), info


class BatchContext:
    """Independent 3D meshes, each with its own material, solved together
    (cfem_create_batch): one set of kernel launches for all instances, with a
    per-instance stopping test. ``problems`` is a list of Problem."""

    def __init__(self, problems, semantics: str = "consistent", stream=None, patch_elems: int = 0,
                 verbose: bool = False):
        self.problems = list(problems)
        n = len(self.problems)
        meshes = (capi.Mesh * n)()
        mats = (capi.Material * n)()
        self._keep = []
        for i, p in enumerate(self.problems):
            if p.dim != 3:
                raise ValueError("batched meshes must be 3D")
            m, k = _mesh_struct(p)
            meshes[i] = m
            mats[i] = capi.Material(float(p.E), float(p.nu), float(p.rho))
            self._keep.append(k)
        opt = capi.Options({"compat": capi.COMPAT, "consistent": capi.CONSISTENT}[semantics], capi.FORM_AUTO,
                           int(patch_elems), int(verbose))
        h = C.c_void_p()
        st = capi.lib().cfem_create_batch(C.byref(h), n, meshes, mats, C.byref(opt), stream)
        capi.check(st, "cfem_create_batch")
        self._h = h
        self.n = n
        self.node_off = np.zeros(n + 1, np.int64)
        self.elem_off = np.zeros(n + 1, np.int64)
        cnt = C.c_int32(0)
        capi.check(capi.lib().cfem_batch_info(self._h, C.byref(cnt), self.node_off.ctypes.data,
                                              self.elem_off.ctypes.data), "cfem_batch_info")

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().cfem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def static_solve(self, precision="fp32_refine", tol=1e-4, stop_rule="residual", max_iter=1000000,
                     outer_tol=1e-10, max_outer=50, allow_not_converged=False):
        """Every instance under its own loads; returns ([u_i [n_nodes_i, 3]], [info_i])."""
        u = np.zeros(int(self.node_off[-1]) * 3, np.float64)
        prm = FemContext._params(precision, tol, stop_rule, max_iter, outer_tol, max_outer)
        infos = (capi.SolveInfo * self.n)()
        st = capi.lib().cfem_batch_static_solve(self._h, C.byref(prm), u.ctypes.data, infos)
        capi.check(st, "cfem_batch_static_solve",
                   (capi.OK, capi.ERR_NOT_CONVERGED) if allow_not_converged else (capi.OK,))
        us = [u[3 * self.node_off[i]:3 * self.node_off[i + 1]].reshape(-1, 3) for i in range(self.n)]
        return us, [FemContext._info(i) for i in infos]

