"""ctypes front-end of the FP64 CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: the GPU solver is tested against it.  Only tests/, the smoke
check in __graft_entry__ and bench.py's CPU-baseline leg may use it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


class Geom(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "otf_size", "pupil_pixels", "patch_size", "n_modes", "n_objects", "n_images",
        "n_channels", "tilt_x", "tilt_y", "n_free", "cutout_size", "pad")]


class Cfg(C.Structure):
    _fields_ = [("n_initial_modes", C.c_int32), ("n_mode_increment", C.c_int32),
                ("max_iterations", C.c_int32), ("min_iterations", C.c_int32),
                ("target_iterations", C.c_int32), ("fd_first", C.c_int32),
                ("ftol", C.c_double), ("eps", C.c_double), ("brent_tol", C.c_double)]


class Report(C.Structure):
    _fields_ = [("initial_metric", C.c_double), ("final_metric", C.c_double),
                ("iterations", C.c_int32), ("status", C.c_int32), ("n_f_evals", C.c_int32),
                ("n_df_evals", C.c_int32), ("fail_count", C.c_int32), ("n_metrics", C.c_int32)]


def build():
    """Compile liboracle.so in place (gcc, optional OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(os.path.join(_HERE, "oracle.c")):
            build()
        L = C.CDLL(path)
        L.orc_fft2.argtypes = [f64p, C.c_int, C.c_int, C.c_int]
        L.orc_reorder.argtypes = [f64p, C.c_int, C.c_int, C.c_int]
        L.orc_autocorrelate.argtypes = [f64p, C.c_int, C.c_int, C.c_int]
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(Geom), f64p, f64p, C.c_int, i32p, C.c_int, i32p,
                                 i32p, i32p, f64p, f64p, f64p, f64p, f64p,
                                 C.c_long, i32p, i32p, f64p, C.c_void_p]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_images.argtypes = [C.c_void_p, f32p, f64p, C.c_void_p]
        L.orc_metric.restype = C.c_double
        L.orc_metric.argtypes = [C.c_void_p, f64p]
        L.orc_gradient.restype = C.c_double
        L.orc_gradient.argtypes = [C.c_void_p, f64p, C.c_void_p, C.c_int, f64p]
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [C.c_void_p, C.POINTER(Cfg), f64p, C.POINTER(Report),
                                C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        for nm in ("orc_get_D", "orc_get_otf", "orc_get_pf", "orc_get_ftsum", "orc_get_gamma",
                   "orc_get_otfnorm"):
            getattr(L, nm).argtypes = [C.c_void_p, f64p]
        L.orc_get_pq.argtypes = [C.c_void_p, f64p, f64p]
        L.orc_get_stats.argtypes = [C.c_void_p, f64p, f64p, f64p]
        L.orc_get_shifts.argtypes = [C.c_void_p, i32p, f64p]
        L.orc_shift.argtypes = [C.c_void_p, f64p]
        L.orc_reorder_into.restype = C.c_int
        L.orc_reorder_into.argtypes = [f64p, C.c_int, C.c_int, f64p, C.c_int, C.c_int, C.c_int]
        L.orc_cons_apply.argtypes = [C.c_void_p, f64p, f64p]
        L.orc_set_fast_fft.argtypes = [C.c_int]
        L.orc_cons_reverse_add.argtypes = [C.c_void_p, f64p, f64p, f64p]
        L.orc_restore.restype = C.c_int
        L.orc_restore.argtypes = [C.c_void_p, f64p, f64p, C.c_int, f64p]
        L.orc_set_fit_plane.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_initial_alpha.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_set_reg_alpha.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_get_plane.argtypes = [C.c_void_p, f32p]
        L.orc_cg_minimize.restype = C.c_int
        L.orc_cg_minimize.argtypes = [C.c_int, C.c_int, C.POINTER(Cfg), C.c_double, F_CB, DF_CB, SHIFT_CB,
                                      C.c_void_p, f64p, C.POINTER(Report), C.c_void_p, C.c_int]
        _LIB = L
    return _LIB


# callbacks of orc_cg_minimize (and of the compiled reference minimiser in oracle/_ref)
F_CB = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_void_p)
DF_CB = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.c_int32, C.c_int32, C.POINTER(C.c_double), C.c_void_p)
SHIFT_CB = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.c_void_p)


def _wrap_callbacks(n_free, f, df, shift):
    def cf(x, _u):
        return float(f(np.ctypeslib.as_array(x, (n_free,)).copy()))

    def cdf(x, method, mc, g, _u):
        out = np.asarray(df(np.ctypeslib.as_array(x, (n_free,)).copy(), int(method), int(mc)), np.float64)
        np.ctypeslib.as_array(g, (n_free,))[:] = out

    def csh(x, _u):
        if shift is not None:
            shift(np.ctypeslib.as_array(x, (n_free,)).copy())

    return F_CB(cf), DF_CB(cdf), SHIFT_CB(csh)


class RefCfg(C.Structure):
    _fields_ = [("mode_start", C.c_int32), ("mode_step", C.c_int32), ("max_iterations", C.c_int32),
                ("min_iterations", C.c_int32), ("target_iterations", C.c_int32), ("fd_first", C.c_int32),
                ("ftol", C.c_double), ("eps", C.c_double)]


_REF = None
REF_PATH = os.path.join(_HERE, "_ref", "libref_cg.so")


def ref_available() -> bool:
    """Whether the reference's own compiled minimiser (oracle/_ref/libref_cg.so) is there; it
    is built from the reference's sources by `make -C oracle ref` (build() does this when the
    reference tree is present)."""
    return os.path.exists(REF_PATH)


def build_ref() -> bool:
    """Builds oracle/_ref/libref_cg.so when the reference tree is present; returns whether the
    library exists afterwards."""
    r = subprocess.run(["make", "-s", "-C", _HERE, "ref"], capture_output=True, text=True)
    return r.returncode == 0 and ref_available()


def ref_lib():
    global _REF
    if _REF is None:
        L = C.CDLL(REF_PATH)
        L.ref_cg_minimize.restype = C.c_int
        L.ref_cg_minimize.argtypes = [C.c_int32, C.c_int32, C.POINTER(RefCfg), C.c_double, F_CB, DF_CB, SHIFT_CB,
                                      C.c_void_p, f64p, C.POINTER(Report), C.c_void_p, C.c_int32]
        _REF = L
    return _REF


def ref_cg_minimize(n_free, n_modes, cfg, grad_scale, f, df, shift=None, cap_metrics=100000):
    """The reference's compiled conjugate_rdx minimiser with its bracket and brent
    (src/lib/util/gsl/conjugate_gradient.cpp, src/lib/math/helpers.cpp) under the Solver::run
    stage loop, on callbacks as cg_minimize.  cfg: an oracle Cfg (brent_tol is the reference's
    fixed 0.1)."""
    rc = RefCfg(mode_start=cfg.n_initial_modes, mode_step=cfg.n_mode_increment, max_iterations=cfg.max_iterations,
                min_iterations=cfg.min_iterations, target_iterations=cfg.target_iterations, fd_first=cfg.fd_first,
                ftol=cfg.ftol, eps=cfg.eps)
    cbs = _wrap_callbacks(n_free, f, df, shift)
    x = np.zeros(n_free)
    rep = Report()
    metrics = np.zeros(cap_metrics)
    ref_lib().ref_cg_minimize(n_free, n_modes, C.byref(rc), grad_scale, cbs[0], cbs[1], cbs[2], None, x,
                              C.byref(rep), metrics.ctypes.data, cap_metrics)
    return dict(x=x, report=rep, metrics=metrics[:min(rep.n_metrics, cap_metrics)].copy())


def cg_minimize(n_free, n_modes, cfg, grad_scale, f, df, shift=None, cap_metrics=100000):
    """The oracle's sequential Solver::run + conjugate_rdx on callbacks (orc_cg_minimize):
    f(x) -> metric, df(x, method, mode_count) -> gradient (method 1 finite differences, 2 Vogel),
    shift(x) between mode stages.  Returns the final x, the report and the metric history."""
    cbs = _wrap_callbacks(n_free, f, df, shift)
    x = np.zeros(n_free)
    rep = Report()
    metrics = np.zeros(cap_metrics)
    lib().orc_cg_minimize(n_free, n_modes, C.byref(cfg), grad_scale, cbs[0], cbs[1], cbs[2], None, x,
                          C.byref(rep), metrics.ctypes.data, cap_metrics)
    return dict(x=x, report=rep, metrics=metrics[:min(rep.n_metrics, cap_metrics)].copy())


def fft2(a: np.ndarray, sign: int = -1) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex128)
    buf = a.view(np.float64).copy()
    lib().orc_fft2(buf, a.shape[0], a.shape[1], sign)
    return buf.view(np.complex128).reshape(a.shape)


def reorder(a: np.ndarray) -> np.ndarray:
    if np.iscomplexobj(a):
        buf = np.ascontiguousarray(a, np.complex128).view(np.float64).copy()
        lib().orc_reorder(buf, a.shape[0], a.shape[1], 1)
        return buf.view(np.complex128).reshape(a.shape)
    buf = np.ascontiguousarray(a, np.float64).copy()
    lib().orc_reorder(buf, a.shape[0], a.shape[1], 0)
    return buf


def reorder_into(a: np.ndarray, out_shape=None, center: bool = False) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float64)
    oy, ox = out_shape if out_shape is not None else a.shape
    out = np.zeros((oy, ox))
    r = lib().orc_reorder_into(a, a.shape[0], a.shape[1], out, oy, ox, int(center))
    if r:
        raise ValueError("reorderInto: target smaller than source")
    return out


def autocorrelate(a: np.ndarray, center: bool = False) -> np.ndarray:
    buf = np.ascontiguousarray(a, np.float64).copy()
    lib().orc_autocorrelate(buf, a.shape[0], a.shape[1], int(center))
    return buf


def default_cfg(max_iterations=50, n_initial_modes=None, n_modes=None, min_iterations=None,
                ftol=0.0, eps=1e-10, target_iterations=3, n_mode_increment=5, fd_first=1):
    """Solver settings; ``max_iterations`` fixed iterations with FTOL = 0 by default."""
    if n_initial_modes is None:
        n_initial_modes = n_modes
    return Cfg(n_initial_modes=n_initial_modes, n_mode_increment=n_mode_increment,
               max_iterations=max_iterations,
               min_iterations=max_iterations if min_iterations is None else min_iterations,
               target_iterations=target_iterations, fd_first=fd_first, ftol=ftol, eps=eps,
               brent_tol=0.1)


def set_fast_fft(on: bool) -> None:
    """Selects the transform of every later solve: the recursive FFT of the oracle proper
    (False, the default) or the iterative Stockham form with precomputed tables (True; the
    same factorisation, rounded differently), which bench.py's CPU baseline times."""
    lib().orc_set_fast_fft(1 if on else 0)


class OraclePatch:
    """One patch of a job in the FP64 oracle."""

    def __init__(self, job, threads: int = 1):
        L = lib()
        self.job = job
        g = Geom(otf_size=job.otf_size, pupil_pixels=job.pupil_pixels, patch_size=job.patch_size,
                 n_modes=job.n_modes, n_objects=job.n_objects, n_images=job.n_images,
                 n_channels=job.n_channels, tilt_x=job.tilt_x, tilt_y=job.tilt_y,
                 n_free=job.nullspace.n_free, cutout_size=job.cutout_size, pad=0)
        self._keep = []
        sup = job.support

        def c(a, dt):
            a = np.ascontiguousarray(a, dt)
            self._keep.append(a)
            return a

        J = c(job.J_T_xy.ravel(), np.float64)
        self.h = L.orc_create(C.byref(g), c(job.modes, np.float64), c(job.pupil, np.float64),
                              int(sup.pupil_support.size), c(sup.pupil_support, np.int32),
                              int(sup.otf_support.size), c(sup.otf_support, np.int32),
                              c(job.img_object, np.int32), c(job.img_channel, np.int32),
                              c(job.phi_fixed, np.float64), c(job.obj_weight, np.float64),
                              c(job.obj_grad_step, np.float64), c(job.window, np.float64),
                              c(job.noise_window, np.float64), int(job.nullspace.vals.size),
                              c(job.nullspace.rows, np.int32), c(job.nullspace.cols, np.int32),
                              c(job.nullspace.vals, np.float64), J.ctypes.data)
        L.orc_set_threads(self.h, threads)
        self.N, self.n = job.otf_size, job.pupil_pixels
        self.I, self.M, self.nObj = job.n_images, job.n_modes, job.n_objects

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_fit_plane(self, on=True):
        """RF_FIT_PLANE: fit and remove each object's mean-image plane (call before set_images)."""
        lib().orc_set_fit_plane(self.h, int(bool(on)))

    def set_initial_alpha(self, alpha=None):
        """Warm start (INIT_FILES): the initial coefficients [I][M] (None: start at zero); the
        next set_images shifts the cutouts by their tilts, solve starts from them."""
        if alpha is None:
            lib().orc_set_initial_alpha(self.h, None)
            return
        self._init = np.ascontiguousarray(alpha, np.float64).ravel()
        lib().orc_set_initial_alpha(self.h, self._init.ctypes.data)

    def set_reg_alpha(self, weights=None):
        """REG_ALPHA: the per-parameter weights [I][M] of 0.5 sum alpha^2 w (None: off)."""
        if weights is None:
            lib().orc_set_reg_alpha(self.h, None)
            return
        self._regw = np.ascontiguousarray(weights, np.float64).ravel()
        lib().orc_set_reg_alpha(self.h, self._regw.ctypes.data)

    def plane(self):
        """The fitted planes [nObj][ps][ps] (float32)."""
        ps = self.job.patch_size
        out = np.zeros((self.nObj, ps, ps), np.float32)
        lib().orc_get_plane(self.h, out)
        return out

    def set_images(self, cutouts, residual_alpha=None, fixed_gamma=None):
        cut = np.ascontiguousarray(cutouts, np.float32)
        ra = np.ascontiguousarray(residual_alpha if residual_alpha is not None
                                  else np.zeros((self.I, 2)), np.float64)
        fg = None
        if fixed_gamma is not None:
            fg = np.ascontiguousarray(fixed_gamma, np.float64)
            self._fg = fg
        lib().orc_set_images(self.h, cut, ra, fg.ctypes.data if fg is not None else None)

    def metric(self, alpha) -> float:
        return lib().orc_metric(self.h, np.ascontiguousarray(alpha, np.float64).ravel())

    def gradient(self, alpha, method="vogel", enabled=None):
        g = np.zeros(self.I * self.M)
        en = None
        if enabled is not None:
            en = np.ascontiguousarray(enabled, np.uint8)
        f = lib().orc_gradient(self.h, np.ascontiguousarray(alpha, np.float64).ravel(),
                               en.ctypes.data if en is not None else None,
                               2 if method == "vogel" else 1, g)
        return f, g.reshape(self.I, self.M)

    def solve(self, cfg, log_evals=False, cap=200000):
        alpha = np.zeros(self.I * self.M)
        rep = Report()
        metrics = np.zeros(100000)
        ev = np.zeros(2 * cap) if log_evals else None
        lib().orc_solve(self.h, C.byref(cfg), alpha, C.byref(rep), metrics.ctypes.data, metrics.size,
                        ev.ctypes.data if ev is not None else None, cap if log_evals else 0)
        out = dict(alpha=alpha.reshape(self.I, self.M), report=rep,
                   metrics=metrics[:rep.n_metrics].copy())
        if log_evals:
            out["evals"] = ev.reshape(-1, 2)
        return out

    def _get(self, name, shape, cplx=False):
        n = int(np.prod(shape)) * (2 if cplx else 1)
        buf = np.zeros(n)
        getattr(lib(), name)(self.h, buf)
        return (buf.view(np.complex128) if cplx else buf).reshape(shape)

    def D(self):
        return self._get("orc_get_D", (self.I, self.N, self.N), True)

    def otf(self):
        return self._get("orc_get_otf", (self.I, self.N, self.N), True)

    def pf(self):
        return self._get("orc_get_pf", (self.I, self.n, self.n), True)

    def ftsum(self):
        return self._get("orc_get_ftsum", (self.nObj, self.N, self.N))

    def gamma(self):
        return self._get("orc_get_gamma", (self.nObj,))

    def otfnorm(self):
        return self._get("orc_get_otfnorm", (self.job.n_channels,))

    def pq(self):
        P = np.zeros(self.nObj * self.N * self.N * 2)
        Q = np.zeros(self.nObj * self.N * self.N)
        lib().orc_get_pq(self.h, P, Q)
        return P.view(np.complex128).reshape(self.nObj, self.N, self.N), Q.reshape(self.nObj, self.N, self.N)

    def cons_reverse_add(self, beta, offset):
        out = np.zeros(self.I * self.M)
        lib().orc_cons_reverse_add(self.h, np.ascontiguousarray(beta, np.float64),
                                   np.ascontiguousarray(offset, np.float64).ravel(), out)
        return out

    def cons_apply(self, galpha):
        out = np.zeros(self.job.nullspace.n_free)
        lib().orc_cons_apply(self.h, np.ascontiguousarray(galpha, np.float64).ravel(), out)
        return out

    def shift(self, alpha):
        lib().orc_shift(self.h, np.ascontiguousarray(alpha, np.float64).ravel())

    def shifts(self):
        s = np.zeros(2 * self.I, np.int32)
        t = np.zeros(2 * self.I)
        lib().orc_get_shifts(self.h, s, t)
        return s.reshape(self.I, 2), t.reshape(self.I, 2)

    def restore(self, alpha, frequency_cutoff, no_filter=False):
        """Restored objects [nObj][ps][ps] at alpha (Object::restorePatch)."""
        fc = np.ascontiguousarray(np.broadcast_to(np.asarray(frequency_cutoff, np.float64), (self.nObj,)))
        out = np.zeros(self.nObj * self.job.patch_size * self.job.patch_size)
        lib().orc_restore(self.h, np.ascontiguousarray(alpha, np.float64).ravel(), fc, int(bool(no_filter)), out)
        return out.reshape(self.nObj, self.job.patch_size, self.job.patch_size)

    def stats(self):
        m, s, n = np.zeros(self.I), np.zeros(self.I), np.zeros(self.I)
        lib().orc_get_stats(self.h, m, s, n)
        return m, s, n
