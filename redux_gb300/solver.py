"""Python mirror of redux's ``momfbd::Solver`` over the GB300 solver core.

The reference interface (include/redux/momfbd/solver.hpp:86-179) is a C++ object built once
per job (``Solver(MomfbdJob&, io_service&, nThreads)``) whose ``run(PatchData::Ptr)``
solves one patch.  Here one ``Solver`` holds the job's static data on the GPU and solves a
batch of patches per ``run``; ``metric``/``gradient`` expose the reference's metric and
gradient evaluations (``Solver::metric``, ``Solver::gradient``) for whole batches.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib


class SolverError(RuntimeError):
    pass


@dataclass
class SolveSettings:
    """GlobalCfg fields read by Solver::run (defaults of config.cpp:629-636)."""
    mode_start: int = 5
    mode_step: int = 5
    max_iterations: int = 500
    min_iterations: int = 5
    target_iterations: int = 3
    fd_first: bool = True
    ftol: float = 1e-3
    eps: float = 1e-10
    max_metrics: int = 1024
    check_every: int = 8

    def to_c(self) -> _lib.SolveParams:
        return _lib.SolveParams(mode_start=self.mode_start, mode_step=self.mode_step,
                                max_iterations=self.max_iterations, min_iterations=self.min_iterations,
                                target_iterations=self.target_iterations, fd_first=int(self.fd_first),
                                max_metrics=self.max_metrics, check_every=self.check_every,
                                ftol=self.ftol, eps=self.eps)


def fixed_iterations(n_modes: int, iterations: int, **kw) -> SolveSettings:
    """All modes at once, exactly `iterations` CG iterations (FTOL = 0)."""
    return SolveSettings(mode_start=n_modes, mode_step=n_modes, max_iterations=iterations,
                         min_iterations=iterations, ftol=0.0, **kw)


class Solver:
    """Batched per-patch MOMFBD solver for one job on one GPU."""

    def __init__(self, job, max_patches: int, precision: str = "fp32", device: int = 0, eval_chunk: int = 0):
        L = _lib.load()
        self.job = job
        self._keep = []

        def c(a, dt):
            a = np.ascontiguousarray(a, dt)
            self._keep.append(a)
            return _lib.ptr(a)

        sup = job.support
        ns = job.nullspace
        self.geo = _lib.Geometry(
            otf_size=job.otf_size, pupil_pixels=job.pupil_pixels, patch_size=job.patch_size,
            n_modes=job.n_modes, n_objects=job.n_objects, n_images=job.n_images, n_channels=job.n_channels,
            tilt_x=job.tilt_x, tilt_y=job.tilt_y, n_free=ns.n_free, cutout_size=job.cutout_size,
            max_patches=max_patches, precision=_lib.RDXG_FP64 if precision == "fp64" else _lib.RDXG_FP32,
            device=device, eval_chunk=eval_chunk)
        st = _lib.Static(
            modes=c(job.modes, np.float64), pupil=c(job.pupil, np.float64),
            n_pupil_support=int(sup.pupil_support.size), pupil_support=c(sup.pupil_support, np.int32),
            n_otf_support=int(sup.otf_support.size), otf_support=c(sup.otf_support, np.int32),
            image_object=c(job.img_object, np.int32), image_channel=c(job.img_channel, np.int32),
            phi_fixed=c(job.phi_fixed, np.float64), object_weight=c(job.obj_weight, np.float64),
            object_grad_step=c(job.obj_grad_step, np.float64), window=c(job.window, np.float64),
            noise_window=c(job.noise_window, np.float64), ns_nnz=int(ns.vals.size),
            ns_rows=c(ns.rows, np.int32), ns_cols=c(ns.cols, np.int32), ns_vals=c(ns.vals, np.float64),
            tilt_jacobian=c(np.asarray(job.J_T_xy).ravel(), np.float64))
        h = C.c_void_p()
        r = L.rdxg_create(C.byref(self.geo), C.byref(st), C.byref(h))
        self.h = h
        self._check(r, "rdxg_create")
        self.precision = precision
        self.max_patches = max_patches
        self.P = 0
        self.I, self.M = job.n_images, job.n_modes

    def _check(self, r, what):
        if r != _lib.RDXG_OK:
            msg = _lib.load().rdxg_last_error(self.h).decode() if self.h else ""
            raise SolverError(f"{what} failed with status {r}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            _lib.load().rdxg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, cuda_stream_ptr: int | None):
        self._check(_lib.load().rdxg_set_stream(self.h, C.c_void_p(cuda_stream_ptr or 0)), "rdxg_set_stream")

    def set_fit_plane(self, enable: bool = True) -> None:
        """FIT_PLANE: remove each object's fitted mean-image plane before windowing and add it
        back to the restored objects (rdxg_set_fit_plane)."""
        self._check(_lib.load().rdxg_set_fit_plane(self.h, int(bool(enable))), "rdxg_set_fit_plane")

    def set_patches(self, cutouts, residual_alpha=None, fixed_gamma=None):
        """cutouts: (P, I, cs, cs) float32 host array or an int device pointer with n_patches."""
        cut = np.ascontiguousarray(cutouts, np.float32)
        P = cut.shape[0]
        ra = None if residual_alpha is None else np.ascontiguousarray(residual_alpha, np.float64)
        fg = None if fixed_gamma is None else np.ascontiguousarray(fixed_gamma, np.float64)
        self._check(_lib.load().rdxg_set_patches(self.h, P, _lib.ptr(cut), _lib.ptr(ra), _lib.ptr(fg)),
                    "rdxg_set_patches")
        self.P = P

    def set_patches_device(self, n_patches: int, dev_ptr: int, residual_alpha=None, fixed_gamma=None):
        ra = None if residual_alpha is None else np.ascontiguousarray(residual_alpha, np.float64)
        fg = None if fixed_gamma is None else np.ascontiguousarray(fixed_gamma, np.float64)
        self._check(_lib.load().rdxg_set_patches_device(self.h, n_patches, C.c_void_p(dev_ptr), _lib.ptr(ra),
                                                        _lib.ptr(fg)), "rdxg_set_patches_device")
        self.P = n_patches

    def set_patch_shapes(self, shapes, patch_shape) -> None:
        """Ragged batch (rdxg_set_patch_shapes): shapes = [(frames, n_modes, nullspace)] with
        each geometry's null space (jobsetup.NullSpace, rows image * n_modes + mode over its
        own images), patch_shape[p] the index of patch p's shape; the next set_patches loads
        len(patch_shape) patches, each with its images in the first slots.  Empty shapes:
        uniform batches again."""
        L = _lib.load()
        if not shapes:
            self._check(L.rdxg_set_patch_shapes(self.h, 0, None, 0, None), "rdxg_set_patch_shapes")
            return
        keep = []
        arr = (_lib.PatchShape * len(shapes))()
        for k, (frames, n_modes, ns) in enumerate(shapes):
            rows = np.ascontiguousarray(ns.rows, np.int32)
            cols = np.ascontiguousarray(ns.cols, np.int32)
            vals = np.ascontiguousarray(ns.vals, np.float64)
            keep += [rows, cols, vals]
            arr[k] = _lib.PatchShape(int(frames), int(n_modes), int(ns.n_free), int(vals.size), _lib.ptr(rows),
                                     _lib.ptr(cols), _lib.ptr(vals))
        ps = np.ascontiguousarray(patch_shape, np.int32)
        self._check(L.rdxg_set_patch_shapes(self.h, len(shapes), arr, int(ps.size), _lib.ptr(ps)),
                    "rdxg_set_patch_shapes")

    def set_reg_alpha(self, weights=None) -> None:
        """REG_ALPHA: weights [I][M] of 0.5 sum alpha^2 w added to the metric (None: off);
        jobsetup.reg_alpha_weights gives the reference's."""
        if weights is None:
            self._check(_lib.load().rdxg_set_reg_alpha(self.h, None), "rdxg_set_reg_alpha")
            return
        w = np.ascontiguousarray(weights, np.float64).reshape(self.I, self.M)
        self._check(_lib.load().rdxg_set_reg_alpha(self.h, _lib.ptr(w)), "rdxg_set_reg_alpha")

    def set_initial_alpha(self, alpha=None) -> None:
        """Warm start: initial coefficients [P][I][M] of the loaded patches (None: zero); the
        images are re-cut by their tilts and every following solve starts there."""
        if alpha is None:
            self._check(_lib.load().rdxg_set_initial_alpha(self.h, None), "rdxg_set_initial_alpha")
            return
        a = np.ascontiguousarray(alpha, np.float64).reshape(self.P, self.I, self.M)
        self._check(_lib.load().rdxg_set_initial_alpha(self.h, _lib.ptr(a)), "rdxg_set_initial_alpha")

    def set_recompute(self, on: bool = True) -> None:
        """Recomputed transforms (rdxg_set_recompute): the gradient kernels form PF, X (and on
        the fused path the OTF) again instead of keeping them per image."""
        self._check(_lib.load().rdxg_set_recompute(self.h, int(bool(on))), "rdxg_set_recompute")

    def recompute(self) -> bool:
        return bool(_lib.load().rdxg_recompute(self.h))

    def set_start_alpha(self, alpha=None) -> None:
        """Continuation: every following solve starts from these coefficients [P][I][M] with the
        images as loaded (not re-cut), e.g. an FP64 handle continuing an FP32 solution."""
        if alpha is None:
            self._check(_lib.load().rdxg_set_start_alpha(self.h, None), "rdxg_set_start_alpha")
            return
        a = np.ascontiguousarray(alpha, np.float64).reshape(self.P, self.I, self.M)
        self._check(_lib.load().rdxg_set_start_alpha(self.h, _lib.ptr(a)), "rdxg_set_start_alpha")

    def metric(self, alpha) -> np.ndarray:
        a = np.ascontiguousarray(alpha, np.float64).reshape(self.P, self.I, self.M)
        out = np.zeros(self.P)
        self._check(_lib.load().rdxg_metric(self.h, _lib.ptr(a), _lib.ptr(out)), "rdxg_metric")
        return out

    def metric_with_reference(self, alpha_ref, alpha) -> np.ndarray:
        """Metric at alpha with the batched metric's reference object taken at alpha_ref."""
        ar = np.ascontiguousarray(alpha_ref, np.float64).reshape(self.P, self.I, self.M)
        a = np.ascontiguousarray(alpha, np.float64).reshape(self.P, self.I, self.M)
        out = np.zeros(self.P)
        self._check(_lib.load().rdxg_metric_with_reference(self.h, _lib.ptr(ar), _lib.ptr(a), _lib.ptr(out)),
                    "rdxg_metric_with_reference")
        return out

    def metric_noalloc(self, alpha) -> np.ndarray:
        """rdxg_metric with every temporary in the library's fixed static device scratch."""
        a = np.ascontiguousarray(alpha, np.float64).reshape(self.P, self.I, self.M)
        out = np.zeros(self.P)
        self._check(_lib.load().rdxg_metric_noalloc(self.h, _lib.ptr(a), _lib.ptr(out)), "rdxg_metric_noalloc")
        return out

    def restore(self, alpha, frequency_cutoff, no_filter: bool = False) -> np.ndarray:
        """Restored objects [P][nObj][ps][ps] at alpha (Object::restorePatch)."""
        a = np.ascontiguousarray(alpha, np.float64).reshape(self.P, self.I, self.M)
        nObj = self.job.n_objects
        fc = np.ascontiguousarray(np.broadcast_to(np.asarray(frequency_cutoff, np.float64), (nObj,)))
        ps = self.job.patch_size
        out = np.zeros((self.P, nObj, ps, ps), np.float32)
        self._check(_lib.load().rdxg_restore(self.h, _lib.ptr(a), _lib.ptr(fc), int(bool(no_filter)), _lib.ptr(out)),
                    "rdxg_restore")
        return out

    def restore_outputs(self, alpha, frequency_cutoff, no_filter: bool = False, psf: str = None,
                        cobj: bool = False, residual: bool = False) -> dict:
        """Restored objects plus the optional outputs of Object::restorePatch
        (rdxg_restore_ex): psf None, "each" ([P][I][ps][ps]) or "mean" ([P][nObj][ps][ps]);
        cobj and residual [P][I][ps][ps]."""
        a = np.ascontiguousarray(alpha, np.float64).reshape(self.P, self.I, self.M)
        nObj, ps = self.job.n_objects, self.job.patch_size
        fc = np.ascontiguousarray(np.broadcast_to(np.asarray(frequency_cutoff, np.float64), (nObj,)))
        flags = 0
        out = {"objects": np.zeros((self.P, nObj, ps, ps), np.float32)}
        if psf == "each":
            flags |= _lib.RDXG_RESTORE_PSF
            out["psf"] = np.zeros((self.P, self.I, ps, ps), np.float32)
        elif psf == "mean":
            flags |= _lib.RDXG_RESTORE_PSF_AVG
            out["psf"] = np.zeros((self.P, nObj, ps, ps), np.float32)
        elif psf is not None:
            raise ValueError("psf: None, 'each' or 'mean'")
        if cobj:
            flags |= _lib.RDXG_RESTORE_COBJ
            out["cobj"] = np.zeros((self.P, self.I, ps, ps), np.float32)
        if residual:
            flags |= _lib.RDXG_RESTORE_RESIDUAL
            out["residual"] = np.zeros((self.P, self.I, ps, ps), np.float32)
        self._check(_lib.load().rdxg_restore_ex(self.h, _lib.ptr(a), _lib.ptr(fc), int(bool(no_filter)), flags,
                                                _lib.ptr(out["objects"]), _lib.ptr(out.get("psf")),
                                                _lib.ptr(out.get("cobj")), _lib.ptr(out.get("residual"))),
                    "rdxg_restore_ex")
        return out

    def gradient(self, alpha, method: str = "vogel", enabled=None):
        a = np.ascontiguousarray(alpha, np.float64).reshape(self.P, self.I, self.M)
        g = np.zeros((self.P, self.I, self.M))
        m = np.zeros(self.P)
        en = None if enabled is None else np.ascontiguousarray(enabled, np.uint8)
        code = {"vogel": _lib.RDXG_GRAD_VOGEL, "exact": _lib.RDXG_GRAD_EXACT, "fd": _lib.RDXG_GRAD_FD}[method]
        self._check(_lib.load().rdxg_gradient(self.h, _lib.ptr(a), _lib.ptr(en), code, _lib.ptr(g), _lib.ptr(m)),
                    "rdxg_gradient")
        return g, m

    def run(self, settings: SolveSettings):
        """Solver::run for every loaded patch."""
        prm = settings.to_c()
        alpha = np.zeros((self.P, self.I, self.M))
        reps = (_lib.PatchReport * self.P)()
        mets = np.zeros((self.P, max(1, settings.max_metrics)))
        self._check(_lib.load().rdxg_solve(self.h, C.byref(prm), _lib.ptr(alpha), reps, _lib.ptr(mets)), "rdxg_solve")
        return dict(alpha=alpha, reports=list(reps), metrics=mets)

    def run_async(self, settings: SolveSettings):
        self._prm = settings.to_c()
        self._check(_lib.load().rdxg_solve_async(self.h, C.byref(self._prm)), "rdxg_solve_async")

    def fetch(self, max_metrics: int):
        alpha = np.zeros((self.P, self.I, self.M))
        reps = (_lib.PatchReport * self.P)()
        mets = np.zeros((self.P, max(1, max_metrics)))
        self._check(_lib.load().rdxg_fetch_results(self.h, _lib.ptr(alpha), reps, _lib.ptr(mets)), "rdxg_fetch_results")
        return dict(alpha=alpha, reports=list(reps), metrics=mets)

    def profile_kernels(self, reps: int = 5) -> dict:
        """Average ms per launch of each kernel on the loaded batch (CUDA events)."""
        ms = np.zeros(5)
        self._check(_lib.load().rdxg_profile_kernels(self.h, reps, _lib.ptr(ms)), "rdxg_profile_kernels")
        return dict(zip(("forward", "accum", "forward_grad", "adjoint", "fd"), ms.tolist()))

    def autotune(self, reps: int = 3) -> dict:
        """The launch-shape planner on the loaded batch (rdxg_autotune): the shapes kept and the
        measured ms per launch of each candidate."""
        sh = _lib.LaunchShape()
        ms = np.zeros(6)
        self._check(_lib.load().rdxg_autotune(self.h, reps, C.byref(sh), _lib.ptr(ms)), "rdxg_autotune")
        return dict(shape=self.launch_shape(), ms=dict(eval=ms[0:2].tolist(), forward=ms[2:4].tolist(),
                                                       adjoint=ms[4:6].tolist()))

    def set_launch_shape(self, eval_threads: int = 0, forward_threads: int = 0, adjoint_threads: int = 0,
                         eval_radix: int = 0, forward_radix: int = 0, adjoint_radix: int = 0,
                         solver_form: int = 0) -> None:
        """Pins the threads per block and the radix plans (first radix) of k_eval, k_forward
        and k_adjoint, and the solver kernel's form (1 staged in shared memory, 2 global
        memory); 0 keeps."""
        sh = _lib.LaunchShape(eval_threads, forward_threads, adjoint_threads, eval_radix, forward_radix, adjoint_radix,
                              solver_form)
        self._check(_lib.load().rdxg_set_launch_shape(self.h, C.byref(sh)), "rdxg_set_launch_shape")

    def launch_shape(self) -> dict:
        """Threads per block (eval, forward, adjoint) and first radix of the transforms'
        plans (eval_radix, ...) in use."""
        sh = _lib.LaunchShape()
        self._check(_lib.load().rdxg_get_launch_shape(self.h, C.byref(sh)), "rdxg_get_launch_shape")
        return dict(eval=sh.eval_threads, forward=sh.forward_threads, adjoint=sh.adjoint_threads,
                    eval_radix=sh.eval_radix, forward_radix=sh.forward_radix, adjoint_radix=sh.adjoint_radix,
                    solver_form=sh.solver_form)

    def launch_count(self) -> int:
        return int(_lib.load().rdxg_last_launch_count(self.h))

    def set_phase_mode(self, mode: int) -> None:
        """Mode expansion of the fused path: 0 CUDA cores (FP32), 2 tensor cores with the
        3xBF16 split, 3 tensor cores with the 6xBF16 split (rdxg_set_phase_mode)."""
        self._check(_lib.load().rdxg_set_phase_mode(self.h, int(mode)), "rdxg_set_phase_mode")

    def phase_mode(self) -> int:
        return int(_lib.load().rdxg_phase_mode(self.h))

    def debug(self, which: str):
        P, I, N, nObj = self.P, self.I, self.job.otf_size, self.job.n_objects
        ct = np.complex128 if self.precision == "fp64" else np.complex64
        spec = {"D": (0, (P, I, N, N), ct), "otf": (1, (P, I, N, N), ct), "gamma": (2, (P, nObj), np.float64),
                "stats": (3, (P, I, 3), np.float64), "object": (4, (P, nObj, N, N), ct),
                "shifts": (5, (P, I, 2), np.int32),
                "phases": (6, (P, I, self.job.pupil_pixels, self.job.pupil_pixels), np.float32),
                "allocations": (7, (1,), np.int64), "allocated_bytes": (8, (1,), np.int64)}[which]
        out = np.zeros(spec[1], spec[2])
        self._check(_lib.load().rdxg_debug_copy(self.h, spec[0], _lib.ptr(out), out.nbytes), "rdxg_debug_copy")
        return out


    def debug_set_tc_status(self, value: int) -> None:
        """Writes the tensor-core expansion's status word (rdxg_debug_set 0), as a bounded wait
        that gave up would leave it."""
        v = np.array([value], np.int32)
        self._check(_lib.load().rdxg_debug_set(self.h, 0, _lib.ptr(v), v.nbytes), "rdxg_debug_set")


def solve_many(solvers, settings: SolveSettings, fetch: bool = True):
    """Solver::run for the loaded patches of several handles (e.g. one per geometry of an
    uneven batch, or one batch split over handles on their own streams) in one CUDA graph
    (rdxg_solve_many); returns each handle's results (None with fetch=False: they stay on
    the device for Solver.fetch)."""
    L = _lib.load()
    hs = (C.c_void_p * len(solvers))(*[s.h for s in solvers])
    prm = settings.to_c()
    r = L.rdxg_solve_many(hs, len(solvers), C.byref(prm))
    if r != _lib.RDXG_OK:
        msgs = "; ".join(L.rdxg_last_error(s.h).decode() for s in solvers)
        raise SolverError(f"rdxg_solve_many failed with status {r}: {msgs}")
    return [s.fetch(settings.max_metrics) for s in solvers] if fetch else None


def cg_minimize(n_free: int, n_modes: int, settings: SolveSettings, grad_scale: float, f, df, shift=None):
    """Host drop-in of the reference's conjugate_rdx + Solver::run stage loop (rdxg_cg_minimize).

    f(x) -> float; df(x, method, mode_count) -> gradient (n_free); shift(x) -> None."""
    L = _lib.load()

    def _f(xp, user):
        return float(f(np.ctypeslib.as_array(xp, shape=(n_free,)).copy()))

    def _df(xp, method, mc, gp, user):
        g = df(np.ctypeslib.as_array(xp, shape=(n_free,)).copy(), int(method), int(mc))
        np.ctypeslib.as_array(gp, shape=(n_free,))[:] = g

    def _sh(xp, user):
        if shift is not None:
            shift(np.ctypeslib.as_array(xp, shape=(n_free,)).copy())

    cf, cdf, csh = _lib.F_FN(_f), _lib.DF_FN(_df), _lib.SHIFT_FN(_sh)
    x = np.zeros(n_free)
    rep = _lib.PatchReport()
    mets = np.zeros(max(1, settings.max_metrics))
    prm = settings.to_c()
    r = L.rdxg_cg_minimize(n_free, n_modes, C.byref(prm), grad_scale, cf, cdf, csh, None, _lib.ptr(x),
                           C.byref(rep), _lib.ptr(mets))
    if r != _lib.RDXG_OK:
        raise SolverError(f"rdxg_cg_minimize failed with status {r}")
    return dict(x=x, report=rep, metrics=mets[:rep.n_metrics].copy())
