"""ctypes binding of ``libsgl_gb300.so`` (declared in ``include/sgl_gb300.h``).

There is no CPU fallback: if the library is missing or no CUDA device is present, every entry
point raises.  Status codes map to the reference's exception types: bad input -> ValueError,
non-finite output -> RuntimeError (sgl_analytic api.py:14-22, 73-74).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().with_name("libsgl_gb300.so")

SGL_OK, SGL_ERR_VALUE, SGL_ERR_CUDA, SGL_ERR_NONFINITE, SGL_ERR_STATE, SGL_ERR_UNSUPPORTED = range(6)
SGL_FP64, SGL_MIXED = 0, 1
PRECISIONS = {"fp64": SGL_FP64, "mixed": SGL_MIXED}

# every symbol the header declares (checked by the CPU test suite)
EXPORTS = ("sgl_abi_version", "sgl_ctx_create", "sgl_ctx_destroy", "sgl_last_error", "sgl_ctx_stream",
           "sgl_ctx_profile", "sgl_stats_json", "sgl_lam_set_cells",
           "sgl_lam_set_xi", "sgl_lam_sigma", "sgl_lnphi", "sgl_xi_term", "sgl_sweep_set_cells", "sgl_sweep_eval", "sgl_measure_peak",
           "sgl_vp_set", "sgl_vp_build", "sgl_vp_lnR", "sgl_invert_opts_default", "sgl_pdf",
           "sgl_gemm_bf16", "sgl_mlp_bias_act", "sgl_mlp_act_grad", "sgl_mlp_col_sum", "sgl_mlp_mse", "sgl_mlp_adamw",
           "sgl_mlp_infer",
           "sgl_plan_grid", "sgl_invert", "sgl_batch_create", "sgl_batch_destroy", "sgl_batch_slots",
           "sgl_batch_slot", "sgl_batch_pdf", "sgl_cfb_set", "sgl_cfb_tune", "sgl_cfb_lnphi", "sgl_cfb_pdf",
           "sgl_cfb_set_separable", "sgl_sur_set", "sgl_sur_judge", "sgl_sur_finish", "sgl_sur_pdf", "sgl_sur_nodes_exact",
           "sgl_cosmo_tables", "sgl_cells_init", "sgl_cells_add", "sgl_cells_xi_init", "sgl_cells_xi_begin",
           "sgl_cells_xi_shear_tail", "sgl_cells_xi_end", "sgl_cells_xi_group", "sgl_cells_read",
           "sgl_cf_kappa_noalloc")


class InvertOpts(C.Structure):
    _fields_ = [("precision", C.c_int), ("tail_box", C.c_int), ("phi_tol", C.c_double),
                ("n_xi_wide", C.c_int), ("n_k_int", C.c_int), ("xi_reach", C.c_double), ("window", C.c_int)]


class Grid(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("nk_k", "nk_g", "n_kap", "n_gam")] + \
               [(n, C.c_double) for n in ("k_k_max", "k_g_max", "kap_min", "kap_max", "gam_max", "sigma",
                                          "phi_at_k_cut", "phi_at_g_cut")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}

    @classmethod
    def from_dict(cls, d):
        g = cls()
        for n, t in cls._fields_:
            setattr(g, n, int(d[n]) if t is C.c_int64 else float(d[n]))
        return g


class InvertMeta(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("nk_k", "nk_g", "n_kap", "n_gam")] + \
               [(n, C.c_double) for n in ("k_k_max", "k_g_max", "kap_min", "kap_max", "gam_max", "xi_min",
                                          "xi_max", "sigma", "phi_at_k_cut", "phi_at_g_cut", "mean", "var",
                                          "skew", "sigmaDL", "norm", "ms_lambda", "ms_transform", "ms_path",
                                          "window", "xi_coarse", "xi_coarse_k")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def lib():
    """Loads the engine library (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH.name} is not built; run `python sgl_analytic_gb300/_build.py` "
                               "(or __graft_entry__.build()) -- there is no CPU fallback")
        L = C.CDLL(str(LIB_PATH))
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int32)
        vp = C.c_void_p
        L.sgl_abi_version.restype = C.c_int
        L.sgl_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
        L.sgl_ctx_destroy.argtypes = [vp]
        L.sgl_ctx_destroy.restype = None
        L.sgl_last_error.argtypes = [vp, C.c_char_p, C.c_int]
        L.sgl_ctx_stream.argtypes = [vp, C.POINTER(vp)]
        L.sgl_ctx_profile.argtypes = [vp, C.c_int]
        L.sgl_stats_json.argtypes = [vp, C.c_char_p, C.c_int, C.c_int]
        L.sgl_stats_json.restype = C.c_int
        L.sgl_lam_set_cells.argtypes = [vp, C.c_int64, dp, dp, dp, ip, dp, C.c_int, C.c_double]
        L.sgl_lam_set_xi.argtypes = [vp, C.c_int, ip, ip, ip, ip, dp, dp, C.c_int, dp, C.c_int, C.c_double,
                                     C.c_double]
        L.sgl_lam_sigma.argtypes = [vp, dp]
        L.sgl_lnphi.argtypes = [vp, dp, C.c_int, dp, C.c_int, C.c_int, dp, dp]
        L.sgl_xi_term.argtypes = [vp, dp, C.c_int, dp, C.c_int, C.c_int, dp, dp]
        L.sgl_sweep_set_cells.argtypes = [vp, C.c_int64, dp, dp]
        L.sgl_sweep_eval.argtypes = [vp, dp, C.c_int, C.c_int, dp, dp]
        L.sgl_measure_peak.argtypes = [vp, C.c_int, dp]
        lp = C.POINTER(C.c_int64)
        L.sgl_vp_set.argtypes = [vp, C.c_int, dp, dp, C.c_int, dp, C.c_int, dp, dp, C.c_int64, ip, dp, C.c_int, lp,
                                 ip, dp, dp, dp, ip, ip, C.c_double]
        L.sgl_vp_lnR.argtypes = [vp, dp, C.c_int, dp, C.c_int, C.c_int, dp, dp]
        L.sgl_vp_build.argtypes = [vp, C.c_int, C.c_int, lp, dp, dp, dp, dp, dp, dp, C.c_double, C.c_double,
                                   C.c_double, dp]
        L.sgl_vp_build.restype = C.c_int
        L.sgl_cfb_set.argtypes = [vp, C.c_int, ip, lp, dp, dp, ip, dp, ip, dp, C.c_int, dp, dp, dp]
        L.sgl_cfb_tune.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.sgl_cfb_lnphi.argtypes = [vp, C.c_int, dp]
        L.sgl_cfb_pdf.argtypes = [vp, C.c_int, dp, C.c_int, dp, C.c_int, dp]
        L.sgl_cfb_set_separable.argtypes = [vp, C.c_int, C.c_int, dp, dp, C.c_int, ip, ip, dp, dp, C.c_int, dp, dp, dp]
        for name in ("sgl_cfb_set", "sgl_cfb_tune", "sgl_cfb_lnphi", "sgl_cfb_pdf", "sgl_cfb_set_separable"):
            getattr(L, name).restype = C.c_int
        L.sgl_sur_set.argtypes = [vp, C.c_int, ip, ip, dp, dp, dp, dp, dp, dp, dp, C.c_int]
        L.sgl_sur_judge.argtypes = [vp, vp, C.c_int, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_float), ip]
        L.sgl_sur_finish.argtypes = [vp, vp, C.c_int, C.c_double, C.c_double, ip, ip]
        L.sgl_sur_pdf.argtypes = [vp, C.c_int, dp, C.c_int, dp, dp]
        L.sgl_sur_nodes_exact.argtypes = [vp, C.c_int, ip, ip, vp, C.c_int, C.c_double, C.c_double]
        L.sgl_cosmo_tables.argtypes = [vp, C.c_int, dp, C.c_int, dp, C.c_int, dp, C.c_int, dp] + [dp] * 8
        L.sgl_cosmo_tables.restype = C.c_int
        ub = C.POINTER(C.c_ubyte)
        L.sgl_cells_init.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp, C.c_int, dp, C.c_int, dp, C.c_int, dp,
                                     C.c_double, C.c_double]
        L.sgl_cells_add.argtypes = [vp, C.c_int, lp, dp, dp, dp, dp, ip, dp, ub, dp]
        L.sgl_cells_xi_init.argtypes = [vp, C.c_int, dp, dp, C.c_int, C.c_int]
        L.sgl_cells_xi_begin.argtypes = [vp, C.c_double]
        L.sgl_cells_xi_shear_tail.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double]
        L.sgl_cells_xi_end.argtypes = [vp, C.POINTER(C.c_int)]
        L.sgl_cells_xi_group.argtypes = [vp, C.c_int, ip, ip, ip, ip, dp, dp, dp]
        L.sgl_cells_read.argtypes = [vp, dp, dp, dp, dp]
        for name in ("sgl_cells_init", "sgl_cells_add", "sgl_cells_xi_init", "sgl_cells_xi_begin",
                     "sgl_cells_xi_shear_tail", "sgl_cells_xi_end", "sgl_cells_xi_group", "sgl_cells_read"):
            getattr(L, name).restype = C.c_int
        for name in ("sgl_sur_set", "sgl_sur_judge", "sgl_sur_finish", "sgl_sur_pdf", "sgl_sur_nodes_exact"):
            getattr(L, name).restype = C.c_int
        for name in ("sgl_sweep_set_cells", "sgl_sweep_eval", "sgl_measure_peak"):
            getattr(L, name).restype = C.c_int
        i64, f32 = C.c_int64, C.c_float
        L.sgl_gemm_bf16.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, i64, i64, vp, i64, i64, vp, i64, i64, f32]
        L.sgl_mlp_bias_act.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int]
        L.sgl_mlp_act_grad.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp]
        L.sgl_mlp_col_sum.argtypes = [vp, C.c_int, C.c_int, vp, vp]
        L.sgl_mlp_mse.argtypes = [vp, i64, vp, vp, vp, dp]
        L.sgl_mlp_adamw.argtypes = [vp, i64, vp, vp, vp, vp, f32, f32, f32, f32, f32, C.c_int]
        L.sgl_mlp_infer.argtypes = [vp, C.c_int, vp, C.c_int, C.POINTER(vp), C.POINTER(vp), vp]
        L.sgl_mlp_infer.restype = C.c_int
        for name in ("sgl_gemm_bf16", "sgl_mlp_bias_act", "sgl_mlp_act_grad", "sgl_mlp_col_sum", "sgl_mlp_mse",
                     "sgl_mlp_adamw"):
            getattr(L, name).restype = C.c_int
        L.sgl_cf_kappa_noalloc.argtypes = [vp, C.c_int, vp, vp, C.c_int64, vp, vp, vp]
        L.sgl_cf_kappa_noalloc.restype = C.c_int
        L.sgl_invert_opts_default.argtypes = [C.POINTER(InvertOpts)]
        L.sgl_invert_opts_default.restype = None
        L.sgl_pdf.argtypes = [vp, dp, C.c_int, C.POINTER(InvertOpts), dp, C.POINTER(InvertMeta)]
        L.sgl_plan_grid.argtypes = [vp, C.POINTER(InvertOpts), C.POINTER(Grid)]
        L.sgl_invert.argtypes = [vp, vp, vp, C.c_int, C.POINTER(Grid), dp, C.c_int, C.POINTER(InvertOpts), dp,
                                 C.POINTER(InvertMeta)]
        L.sgl_batch_create.argtypes = [C.c_int, C.c_int, C.POINTER(vp)]
        L.sgl_batch_destroy.argtypes = [vp]
        L.sgl_batch_destroy.restype = None
        L.sgl_batch_slots.argtypes = [vp]
        L.sgl_batch_slots.restype = C.c_int
        L.sgl_batch_slot.argtypes = [vp, C.c_int]
        L.sgl_batch_slot.restype = vp
        L.sgl_batch_pdf.argtypes = [vp, C.c_int, ip, dp, C.c_int, C.POINTER(InvertOpts), dp, C.POINTER(InvertMeta), ip]
        for name in ("sgl_batch_create", "sgl_batch_pdf", "sgl_ctx_create", "sgl_ctx_stream", "sgl_ctx_profile", "sgl_lam_set_cells", "sgl_lam_set_xi", "sgl_lam_sigma", "sgl_lnphi",
                     "sgl_xi_term", "sgl_pdf", "sgl_vp_set", "sgl_vp_lnR", "sgl_plan_grid", "sgl_invert"):
            getattr(L, name).restype = C.c_int
        if L.sgl_abi_version() != 2:
            raise RuntimeError("libsgl_gb300.so ABI version mismatch; rebuild it")
        _lib = L
    return _lib


def _ptr(a, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


def _raise(status, msg):
    if status == SGL_ERR_VALUE:
        raise ValueError(msg)
    if status == SGL_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)


class Engine:
    """One engine context on one CUDA device (own stream and device arena).  With `handle`, a view
    of a context that something else owns (a batch slot): close() then leaves it alone."""

    def __init__(self, device=0, handle=None, owner=None):
        L = lib()
        if handle is not None:
            self._h, self._L, self.device, self._owner = C.c_void_p(handle), L, int(device), owner
            return
        self._owner = None
        h = C.c_void_p()
        st = L.sgl_ctx_create(int(device), C.byref(h))
        if st != SGL_OK:
            buf = C.create_string_buffer(512)
            L.sgl_last_error(None, buf, 512)
            _raise(st, "sgl_ctx_create: " + buf.value.decode())
        self._h = h
        self._L = L
        self.device = int(device)

    def close(self):
        if getattr(self, "_h", None):
            if getattr(self, "_owner", None) is None:
                self._L.sgl_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != SGL_OK:
            buf = C.create_string_buffer(1024)
            self._L.sgl_last_error(self._h, buf, 1024)
            _raise(st, f"{what}: {buf.value.decode()}")

    @property
    def stream(self):
        """The engine's cudaStream_t as an integer handle (for torch.cuda.ExternalStream)."""
        h = C.c_void_p()
        self._check(self._L.sgl_ctx_stream(self._h, C.byref(h)), "sgl_ctx_stream")
        return h.value or 0

    def profile(self, enable=True):
        self._check(self._L.sgl_ctx_profile(self._h, int(bool(enable))), "sgl_ctx_profile")

    def stats(self, reset=False):
        import json
        n = self._L.sgl_stats_json(self._h, None, 0, 0)
        buf = C.create_string_buffer(n + 1)
        self._L.sgl_stats_json(self._h, buf, n + 1, int(bool(reset)))
        return json.loads(buf.value.decode())

    # ---------------------------------------------------------------- population
    def set_cells(self, w0, k0, g0, ig, fe_g, V):
        w0, k0, g0, fe_g = (np.ascontiguousarray(a, np.float64) for a in (w0, k0, g0, fe_g))
        ig = np.ascontiguousarray(ig, np.int32)
        n = w0.size
        if not (k0.size == g0.size == ig.size == n):
            raise ValueError("cell arrays must have equal length")
        self._check(self._L.sgl_lam_set_cells(self._h, n, _ptr(w0), _ptr(k0), _ptr(g0), _ptr(ig, C.c_int32),
                                              _ptr(fe_g), fe_g.size, float(V)), "sgl_lam_set_cells")

    def set_xi(self, m, nrow, nidx, idx, rows, ce_k, ce_g, prune=1e-7, s0=0.0):
        m, nrow, nidx, idx = (np.ascontiguousarray(a, np.int32) for a in (m, nrow, nidx, idx))
        rows, ce_k, ce_g = (np.ascontiguousarray(a, np.float64) for a in (rows, ce_k, ce_g))
        if rows.size != int(np.sum(nrow.astype(np.int64) * (nidx.astype(np.int64) + 1))):
            raise ValueError("rows size does not match nrow x (nidx + 1)")
        if idx.size != int(np.sum(nidx.astype(np.int64))):
            raise ValueError("idx size does not match nidx")
        self._check(self._L.sgl_lam_set_xi(self._h, m.size, _ptr(m, C.c_int32), _ptr(nrow, C.c_int32),
                                           _ptr(nidx, C.c_int32), _ptr(idx, C.c_int32), _ptr(rows), _ptr(ce_k),
                                           ce_k.size, _ptr(ce_g), ce_g.size, float(prune), float(s0)),
                    "sgl_lam_set_xi")

    def sigma(self):
        s = C.c_double()
        self._check(self._L.sgl_lam_sigma(self._h, C.byref(s)), "sgl_lam_sigma")
        return s.value

    def lnphi(self, kk, kg, precision=SGL_FP64):
        kk = np.ascontiguousarray(np.atleast_1d(kk), np.float64)
        kg = np.ascontiguousarray(np.atleast_1d(kg), np.float64)
        re = np.empty((kk.size, kg.size))
        im = np.empty((kk.size, kg.size))
        self._check(self._L.sgl_lnphi(self._h, _ptr(kk), kk.size, _ptr(kg), kg.size, int(precision), _ptr(re),
                                      _ptr(im)), "sgl_lnphi")
        return re + 1j * im

    def xi_term(self, kk, kg, precision=SGL_FP64):
        kk = np.ascontiguousarray(np.atleast_1d(kk), np.float64)
        kg = np.ascontiguousarray(np.atleast_1d(kg), np.float64)
        re = np.empty((kk.size, kg.size))
        im = np.empty((kk.size, kg.size))
        self._check(self._L.sgl_xi_term(self._h, _ptr(kk), kk.size, _ptr(kg), kg.size, int(precision), _ptr(re),
                                        _ptr(im)), "sgl_xi_term")
        return re + 1j * im

    # ---------------------------------------------------------------- batched CF solver
    def cfb_set(self, b):
        """Uploads a batch (a mapping as sgl_analytic_gb300.cfbatch.Batch.arrays() gives)."""
        i32 = lambda a: np.ascontiguousarray(a, np.int32)
        f64 = lambda a: np.ascontiguousarray(a, np.float64)
        self._cfb = dict(inst_plane0=i32(b["inst_plane0"]), plane_cells=np.ascontiguousarray(b["plane_cells"], np.int64),
                         kap=f64(b["kap"]), w=f64(b["w"]), nk=i32(b["nk"]), dk=f64(b["dk"]), closure=i32(b["closure"]),
                         V=f64(b["V"]), vp_D=f64(b["vp_D"]), vp_K=f64(b["vp_K"]), vp_w=f64(b["vp_w"]))
        a = self._cfb
        self._check(self._L.sgl_cfb_set(self._h, a["nk"].size, _ptr(a["inst_plane0"], C.c_int32),
                                        _ptr(a["plane_cells"], C.c_int64), _ptr(a["kap"]), _ptr(a["w"]),
                                        _ptr(a["nk"], C.c_int32), _ptr(a["dk"]), _ptr(a["closure"], C.c_int32),
                                        _ptr(a["V"]), int(b["nstate"]), _ptr(a["vp_D"]), _ptr(a["vp_K"]), _ptr(a["vp_w"])),
                    "sgl_cfb_set")

    def cfb_set_separable(self, F, g, inst_plane0, nk, dk, V, u, v, k0=None, geom=False):
        """Uploads a gauss-closure batch of template planes: plane p's cell (m, b) has kap = u[p, m] F[m, b]
        and w = v[p, m] g[b]; the cells are built on the device.  k0: per-instance offset of the solve's
        k points (k0 + n dk), or with geom their log-spaced form exp(k0 + n dk)."""
        F = np.ascontiguousarray(F, np.float64)
        nm, nb = F.shape
        g = np.ascontiguousarray(g, np.float64)
        i32 = lambda a: np.ascontiguousarray(a, np.int32)
        f64 = lambda a: np.ascontiguousarray(a, np.float64)
        p0, nk, dk, V, u, v = i32(inst_plane0), i32(nk), f64(dk), f64(V), f64(u), f64(v)
        n_planes = int(p0[-1])
        if g.size != nb or u.shape != (n_planes, nm) or v.shape != (n_planes, nm) or nk.size != p0.size - 1 or \
                dk.size != nk.size or V.size != nk.size:
            raise ValueError("separable batch arrays have inconsistent sizes")
        k0 = None if k0 is None else f64(k0)
        if k0 is not None and k0.size != nk.size:
            raise ValueError("k0 needs one entry per instance")
        self._cfb = dict(nk=nk)
        self._check(self._L.sgl_cfb_set_separable(self._h, nm, nb, _ptr(F), _ptr(g), nk.size, _ptr(p0, C.c_int32),
                                                  _ptr(nk, C.c_int32), _ptr(dk), None if k0 is None else _ptr(k0),
                                                  int(bool(geom)), _ptr(V), _ptr(u), _ptr(v)), "sgl_cfb_set_separable")

    def cfb_tune(self, precision=SGL_MIXED):
        kt, cps = C.c_int(), C.c_int()
        self._check(self._L.sgl_cfb_tune(self._h, int(precision), C.byref(kt), C.byref(cps)), "sgl_cfb_tune")
        return kt.value, cps.value

    def cfb_lnphi(self, precision=SGL_MIXED, host=True):
        """ln Phi of every instance, concatenated (complex); host=False leaves it on the device only."""
        if not host:
            self._check(self._L.sgl_cfb_lnphi(self._h, int(precision), None), "sgl_cfb_lnphi")
            return None
        n = int(np.sum(self._cfb["nk"].astype(np.int64)))
        out = np.empty(2 * n)
        self._check(self._L.sgl_cfb_lnphi(self._h, int(precision), _ptr(out)), "sgl_cfb_lnphi")
        return out[0::2] + 1j * out[1::2]

    def cfb_pdf(self, lnmu, precision=SGL_MIXED, use_graph=True):
        """(dP/dln mu [n_inst, n_lnmu], device ms of the step)."""
        x = np.ascontiguousarray(lnmu, np.float64)
        out = np.empty((self._cfb["nk"].size, x.size))
        ms = C.c_double()
        self._check(self._L.sgl_cfb_pdf(self._h, int(precision), _ptr(x), x.size, _ptr(out), int(bool(use_graph)),
                                        C.byref(ms)), "sgl_cfb_pdf")
        return out, ms.value

    # ---------------------------------------------------------------- surrogate + judge sweep
    def sur_set(self, inst_plane0, nk, dk, s, dz, mu1, mu2, lnq0, hq, nq):
        i32 = lambda a: np.ascontiguousarray(a, np.int32)
        f64 = lambda a: np.ascontiguousarray(a, np.float64)
        self._sur = dict(inst_plane0=i32(inst_plane0), nk=i32(nk), dk=f64(dk), s=f64(s), dz=f64(dz), mu1=f64(mu1),
                         mu2=f64(mu2), lnq0=f64(lnq0), hq=f64(hq))
        a = self._sur
        n = int(a["inst_plane0"][-1])
        if not all(a[k].size == n for k in ("s", "dz", "mu1", "mu2", "lnq0", "hq")) or \
                a["nk"].size != a["inst_plane0"].size - 1 or a["dk"].size != a["nk"].size:
            raise ValueError("surrogate sweep arrays have inconsistent sizes")
        self._check(self._L.sgl_sur_set(self._h, a["nk"].size, _ptr(a["inst_plane0"], C.c_int32), _ptr(a["nk"], C.c_int32),
                                        _ptr(a["dk"]), _ptr(a["s"]), _ptr(a["dz"]), _ptr(a["mu1"]), _ptr(a["mu2"]),
                                        _ptr(a["lnq0"]), _ptr(a["hq"]), int(nq)), "sgl_sur_set")

    def sur_judge(self, Y, members, shift, scale, tau):
        """Y: device tensor [members, planes * nq, 2] (float32).  Returns ((n_planes, 2) largest dz |spread|
        per plane, as is and |Phi|-weighted; (n_planes, 2) band [first, end) of k indices whose weighted
        spread exceeds tau, (0, 0) if none)."""
        n = self._sur["s"].size
        out = np.empty(2 * n, np.float32)
        band = np.empty(2 * n, np.int32)
        self._check(self._L.sgl_sur_judge(self._h, C.c_void_p(Y.data_ptr()), int(members), float(shift), float(scale),
                                          float(tau), out.ctypes.data_as(C.POINTER(C.c_float)), _ptr(band, C.c_int32)),
                    "sgl_sur_judge")
        return out.reshape(-1, 2), band.reshape(-1, 2)

    def sur_finish(self, Y, members, shift, scale, exact_inst, exact_lo=None):
        e = np.ascontiguousarray(exact_inst, np.int32)
        lo = None if exact_lo is None else np.ascontiguousarray(exact_lo, np.int32)
        if e.size != self._sur["s"].size or (lo is not None and lo.size != e.size):
            raise ValueError("exact_inst / exact_lo need one entry per plane")
        self._check(self._L.sgl_sur_finish(self._h, C.c_void_p(Y.data_ptr()), int(members), float(shift), float(scale),
                                           _ptr(e, C.c_int32), None if lo is None else _ptr(lo, C.c_int32)),
                    "sgl_sur_finish")

    def sur_nodes_exact(self, planes, Y, members, shift, scale, node_lo=None):
        """Writes the batched solver's node values of `planes` (instance j = planes[j], from node node_lo[j])
        into Y."""
        pl = np.ascontiguousarray(planes, np.int32)
        lo = None if node_lo is None else np.ascontiguousarray(node_lo, np.int32)
        if lo is not None and lo.size != pl.size:
            raise ValueError("node_lo needs one entry per plane")
        self._check(self._L.sgl_sur_nodes_exact(self._h, pl.size, _ptr(pl, C.c_int32),
                                                None if lo is None else _ptr(lo, C.c_int32), C.c_void_p(Y.data_ptr()),
                                                int(members), float(shift), float(scale)), "sgl_sur_nodes_exact")

    def sur_pdf(self, lnmu, precision=SGL_FP64, want_lnphi=False):
        x = np.ascontiguousarray(lnmu, np.float64)
        out = np.empty((self._sur["nk"].size, x.size))
        lp = np.empty(2 * int(np.sum(self._sur["nk"].astype(np.int64)))) if want_lnphi else None
        self._check(self._L.sgl_sur_pdf(self._h, int(precision), _ptr(x), x.size, _ptr(out),
                                        _ptr(lp) if want_lnphi else None), "sgl_sur_pdf")
        return (out, lp[0::2] + 1j * lp[1::2]) if want_lnphi else out

    def vp_build(self, pop, nstate=48, eta=None):
        """Builds and installs the vp closure from its per-shell population (sgl_vp_build): a mapping
        with shell_start, W, kap, gam, phi, rho, fvar, target_kappa, target_gamma.  eta: None to
        calibrate, else the value to use.  Returns eta."""
        ss = np.ascontiguousarray(pop["shell_start"], np.int64)
        W, kap, gam, phi = (np.ascontiguousarray(pop[k], np.float64) for k in ("W", "kap", "gam", "phi"))
        rho, fvar = np.ascontiguousarray(pop["rho"], np.float64), np.ascontiguousarray(pop["fvar"], np.float64)
        ns = ss.size - 1
        if not (W.size == kap.size == gam.size == phi.size == ss[-1]) or rho.size != max(ns - 1, 0) or fvar.size != ns:
            raise ValueError("vp population arrays do not match shell_start")
        out = C.c_double()
        self._check(self._L.sgl_vp_build(self._h, int(nstate), ns, _ptr(ss, C.c_int64), _ptr(W), _ptr(kap), _ptr(gam),
                                         _ptr(phi), _ptr(rho), _ptr(fvar), float(pop["target_kappa"]),
                                         float(pop["target_gamma"]), -1.0 if eta is None else float(eta),
                                         C.byref(out)), "sgl_vp_build")
        return out.value

    def set_vp(self, d):
        """Installs the positive (vp) closure from a mapping with the arrays of sgl_vp_set (u, w, K, ku,
        gu, cu, cw, gstart, sh_g, ga, gb, gc, glo, ghi, shear_var); None removes it."""
        if d is None:
            self._check(self._L.sgl_vp_set(self._h, 48, None, None, 0, None, 0, None, None, 0, None, None, 0, None,
                                           None, None, None, None, None, None, 0.0), "sgl_vp_set")
            return
        f64 = lambda k: np.ascontiguousarray(d[k], np.float64)
        i32 = lambda k: np.ascontiguousarray(d[k], np.int32)
        u, w, ku, gu, cw, ga, gb, gc = (f64(k) for k in ("u", "w", "ku", "gu", "cw", "ga", "gb", "gc"))
        K = np.ascontiguousarray(d["K"], np.float64).reshape(-1)
        cu, sh_g, glo, ghi = (i32(k) for k in ("cu", "sh_g", "glo", "ghi"))
        gstart = np.ascontiguousarray(d["gstart"], np.int64)
        nsh, G = sh_g.size - 1, ga.size
        if u.size != w.size or ku.size != gu.size or cu.size != cw.size or gstart.size != G + 1 or \
                not (gb.size == gc.size == glo.size == ghi.size == G) or K.size != max(nsh - 1, 0) * u.size ** 2:
            raise ValueError("vp closure arrays have inconsistent sizes")
        self._check(self._L.sgl_vp_set(self._h, u.size, _ptr(u), _ptr(w), nsh, _ptr(K), ku.size, _ptr(ku), _ptr(gu),
                                       cu.size, _ptr(cu, C.c_int32), _ptr(cw), G, _ptr(gstart, C.c_int64),
                                       _ptr(sh_g, C.c_int32), _ptr(ga), _ptr(gb), _ptr(gc), _ptr(glo, C.c_int32),
                                       _ptr(ghi, C.c_int32), float(d["shear_var"])), "sgl_vp_set")

    def vp_lnR(self, kv, qv, precision=SGL_FP64):
        kv = np.ascontiguousarray(np.atleast_1d(kv), np.float64)
        qv = np.ascontiguousarray(np.atleast_1d(qv), np.float64)
        re = np.empty((kv.size, qv.size))
        im = np.empty((kv.size, qv.size))
        self._check(self._L.sgl_vp_lnR(self._h, _ptr(kv), kv.size, _ptr(qv), qv.size, int(precision), _ptr(re),
                                       _ptr(im)), "sgl_vp_lnR")
        return re + 1j * im

    def sweep_set_cells(self, kap, w):
        kap = np.ascontiguousarray(kap, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        if kap.size != w.size:
            raise ValueError("kap and w must have equal length")
        self._check(self._L.sgl_sweep_set_cells(self._h, kap.size, _ptr(kap), _ptr(w)), "sgl_sweep_set_cells")

    def sweep(self, kk, precision=SGL_FP64):
        kk = np.ascontiguousarray(np.atleast_1d(kk), np.float64)
        re = np.empty(kk.size)
        im = np.empty(kk.size)
        self._check(self._L.sgl_sweep_eval(self._h, _ptr(kk), kk.size, int(precision), _ptr(re), _ptr(im)),
                    "sgl_sweep_eval")
        return re + 1j * im

    def cosmo_tables(self, params, z, M, zm=()):
        """Tables of n cosmologies (rows of params: h, Om, Ob, s8, ns, zeq, Ok, w0, wa) -- the reference's
        chain Cosmology: dict of E, chi, DM, D at z (n x nz), sigmaM, dlnsig at M (n x nm), dndlnM, conc at
        zm x M (n x nzm x nm)."""
        p = np.ascontiguousarray(np.atleast_2d(params), np.float64)
        if p.shape[1] != 9:
            raise ValueError("params rows are (h, Om, Ob, s8, ns, zeq, Ok, w0, wa)")
        z, M, zm = (np.ascontiguousarray(np.atleast_1d(a), np.float64) for a in (z, M, zm))
        n, nz, nm, nzm = p.shape[0], z.size, M.size, zm.size
        out = {k: np.empty((n, nz)) for k in ("E", "chi", "DM", "D")}
        out.update(sigmaM=np.empty((n, nm)), dlnsig=np.empty((n, nm)), dndlnM=np.empty((n, max(nzm, 1), nm)),
                   conc=np.empty((n, max(nzm, 1), nm)))
        self._check(self._L.sgl_cosmo_tables(self._h, n, _ptr(p), nz, _ptr(z), nm, _ptr(M), nzm,
                                             _ptr(zm) if nzm else None, *[_ptr(out[k]) for k in
                                             ("E", "chi", "DM", "D", "sigmaM", "dlnsig", "dndlnM", "conc")]),
                    "sgl_cosmo_tables")
        if nzm == 0:
            del out["dndlnM"], out["conc"]
        return out

    def measure_peak(self, fp64=True):
        t = C.c_double()
        self._check(self._L.sgl_measure_peak(self._h, int(bool(fp64)), C.byref(t)), "sgl_measure_peak")
        return t.value

    def _opts(self, precision, tail_box, phi_tol, n_xi_wide, n_k_int, xi_reach, window):
        o = InvertOpts()
        self._L.sgl_invert_opts_default(C.byref(o))
        o.precision, o.tail_box, o.phi_tol = int(precision), int(bool(tail_box)), float(phi_tol)
        o.n_xi_wide, o.n_k_int, o.xi_reach = int(n_xi_wide), int(n_k_int), float(xi_reach)
        if window not in (True, False, "auto", None):
            raise ValueError(f"window must be True, False or 'auto', got {window!r}")
        o.window = 2 if window == "auto" else (1 if window is True else 0)
        return o

    def pdf(self, xi_out, precision=SGL_FP64, tail_box=True, phi_tol=1e-8, n_xi_wide=500, n_k_int=2400,
            xi_reach=24.0, window=False):
        x = np.ascontiguousarray(xi_out, np.float64)
        out = np.empty(x.size)
        o = self._opts(precision, tail_box, phi_tol, n_xi_wide, n_k_int, xi_reach, window)
        meta = InvertMeta()
        self._check(self._L.sgl_pdf(self._h, _ptr(x), x.size, C.byref(o), _ptr(out), C.byref(meta)), "sgl_pdf")
        return out, meta.as_dict()

    def plan_grid(self, precision=SGL_FP64, tail_box=True, phi_tol=1e-8, xi_reach=24.0):
        """The inversion grid of the loaded population (sgl_plan_grid): a dict of sgl_grid's fields."""
        o = self._opts(precision, tail_box, phi_tol, 500, 2400, xi_reach, False)
        g = Grid()
        self._check(self._L.sgl_plan_grid(self._h, C.byref(o), C.byref(g)), "sgl_plan_grid")
        return g.as_dict()

    def invert_phi(self, phi, grid, xi_out, precision=SGL_FP64, tail_box=True, phi_tol=1e-8, n_xi_wide=500,
                   n_k_int=2400, xi_reach=24.0, window=False):
        """P_s on xi_out from a caller-owned Phi on `grid` (sgl_invert).  phi: a complex (nk_k, nk_g)
        NumPy array (host), or a pair (re, im) of device pointers (ints) to FP64 planes on this
        engine's device."""
        x = np.ascontiguousarray(xi_out, np.float64)
        out = np.empty(x.size)
        o = self._opts(precision, tail_box, phi_tol, n_xi_wide, n_k_int, xi_reach, window)
        g = Grid.from_dict(grid)
        meta = InvertMeta()
        if isinstance(phi, tuple):
            re_p, im_p, on_dev = C.c_void_p(int(phi[0])), C.c_void_p(int(phi[1])), 1
            keep = None
        else:
            phi = np.asarray(phi)
            if phi.shape != (g.nk_k, g.nk_g):
                raise ValueError(f"Phi has shape {phi.shape}, the grid is {(g.nk_k, g.nk_g)}")
            keep = (np.ascontiguousarray(phi.real, np.float64), np.ascontiguousarray(phi.imag, np.float64))
            re_p, im_p, on_dev = C.c_void_p(keep[0].ctypes.data), C.c_void_p(keep[1].ctypes.data), 0
        self._check(self._L.sgl_invert(self._h, re_p, im_p, on_dev, C.byref(g), _ptr(x), x.size, C.byref(o), _ptr(out),
                                       C.byref(meta)), "sgl_invert")
        del keep
        return out, meta.as_dict()


class Batch:
    """The native batched solver (sgl_batch_*): `slots` contexts on one device and a host thread
    per slot.  slot(i) is an Engine view of slot i's context (load its population through it)."""

    def __init__(self, slots=4, device=0):
        self._L = lib()
        h = C.c_void_p()
        st = self._L.sgl_batch_create(int(device), int(slots), C.byref(h))
        if st != SGL_OK:
            buf = C.create_string_buffer(512)
            self._L.sgl_last_error(None, buf, 512)
            _raise(st, "sgl_batch_create: " + buf.value.decode())
        self._h = h
        self.device = int(device)
        self.engines = [Engine(device, handle=self._L.sgl_batch_slot(h, i), owner=self) for i in range(int(slots))]

    def slot(self, i):
        return self.engines[i]

    def pdf(self, job_slot, xi_out, precision=SGL_FP64, tail_box=True, phi_tol=1e-8, n_xi_wide=500, n_k_int=2400,
            xi_reach=24.0, window=False):
        """Runs one PDF per entry of job_slot (the slot it runs on); returns (P [jobs, n_xi], metas)."""
        js = np.ascontiguousarray(job_slot, np.int32)
        x = np.ascontiguousarray(xi_out, np.float64)
        out = np.empty((js.size, x.size))
        o = self.engines[0]._opts(precision, tail_box, phi_tol, n_xi_wide, n_k_int, xi_reach, window)
        metas = (InvertMeta * max(1, js.size))()
        status = np.zeros(max(1, js.size), np.int32)
        st = self._L.sgl_batch_pdf(self._h, js.size, _ptr(js, C.c_int32), _ptr(x), x.size, C.byref(o), _ptr(out),
                                   metas, _ptr(status, C.c_int32))
        if st != SGL_OK:
            buf = C.create_string_buffer(1024)
            self._L.sgl_last_error(None, buf, 1024)
            _raise(st, buf.value.decode())
        return out, [metas[i].as_dict() for i in range(js.size)]

    def close(self):
        if getattr(self, "_h", None):
            for e in self.engines:
                e._h = None
            self._L.sgl_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
