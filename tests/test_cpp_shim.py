"""The C++ shim include/rdxg_solver.hpp (the shape of redux's momfbd::Solver over the C ABI):
it compiles and links against the library on any host; on a GPU, a batch solved through it
gives the same alpha, metric history, final metric and restored objects as the Python
harness over the same C ABI."""
import os
import subprocess

import numpy as np
import pytest

from redux_gb300 import solver as S
from tests.conftest import workload

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "redux_gb300")


def _build(out_dir):
    from redux_gb300 import build as B
    B.build()
    exe = os.path.join(out_dir, "shim_solve")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_solve.cpp"), "-o", exe,
           "-L", LIBDIR, "-lredux_gb300", "-Wl,-rpath," + LIBDIR]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_shim_compiles_and_links(tmp_path):
    exe = _build(str(tmp_path))
    assert os.path.exists(exe)


def _dump(job, cutouts, fixed_gamma, st, fc, d, save_mask=0, extras=None):
    sup, ns = job.support, job.nullspace
    geom = [job.otf_size, job.pupil_pixels, job.patch_size, job.n_modes, job.n_objects, job.n_images,
            job.n_channels, job.tilt_x, job.tilt_y, ns.n_free, job.cutout_size, cutouts.shape[0], 0, 0]
    arrays = {
        "geom.i32": np.asarray(geom, np.int32), "modes.f64": job.modes, "pupil.f64": job.pupil,
        "pupil_support.i32": sup.pupil_support, "otf_support.i32": sup.otf_support,
        "image_object.i32": job.img_object, "image_channel.i32": job.img_channel,
        "phi_fixed.f64": job.phi_fixed, "object_weight.f64": job.obj_weight,
        "object_grad_step.f64": job.obj_grad_step, "window.f64": job.window,
        "noise_window.f64": job.noise_window, "ns_rows.i32": ns.rows, "ns_cols.i32": ns.cols,
        "ns_vals.f64": ns.vals, "tilt_jacobian.f64": np.asarray(job.J_T_xy).ravel(),
        "settings.f64": [st.mode_start, st.mode_step, st.max_iterations, st.min_iterations,
                         st.target_iterations, float(st.fd_first), st.ftol, st.eps, st.max_metrics,
                         float(save_mask)],
        "fc.f64": np.full(job.n_objects, fc), "cutouts.f32": cutouts,
    }
    if fixed_gamma is not None:
        arrays["fixed_gamma.f64"] = fixed_gamma
    if extras:
        arrays["fit_plane.i32"] = [1]
        arrays["reg_alpha.f64"] = extras["reg_alpha"]
        arrays["init_alpha.f64"] = extras["init_alpha"]
    for name, a in arrays.items():
        dt = {"i32": np.int32, "f64": np.float64, "f32": np.float32}[name.rsplit(".", 1)[1]]
        np.ascontiguousarray(a, dt).tofile(os.path.join(d, name))


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", ["plain64", "production88", "plain64+"])
def test_shim_solve_matches_the_python_harness(tmp_path, cfg, monkeypatch):
    """cfg "plain64+": the plain 64 x 64 workload with FIT_PLANE, REG_ALPHA and a warm start.
    The driver runs in a process of its own, whose launch-shape planner could keep the other
    radix plan (it times the candidates, as FFTW_MEASURE does): both processes keep the default
    shapes (RDXG_AUTOTUNE=0), so that the bits compare."""
    monkeypatch.setenv("RDXG_AUTOTUNE", "0")
    extras = None
    if cfg == "plain64+":
        from redux_gb300 import jobsetup as js
        w = workload("plain64")
        extras = dict(reg_alpha=js.reg_alpha_weights(np.sqrt(w.job.atm_var), w.job.n_images, w.job.patch_size,
                                                     w.job.wavelength, 1e3),
                      init_alpha=w.patches.alpha_true * 0.5)
        cfg = "plain64"
    else:
        w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    job = w.job
    st = S.SolveSettings(mode_start=5, mode_step=5, max_iterations=6, min_iterations=3, ftol=1e-3, max_metrics=128)
    fc = job.otf_size / 2.0
    d = str(tmp_path)
    # per-image PSFs for one configuration, the object means for the other
    from redux_gb300 import _lib
    psf_flag = _lib.RDXG_RESTORE_PSF if cfg == "plain64" else _lib.RDXG_RESTORE_PSF_AVG
    _dump(job, w.patches.cutouts, w.patches.fixed_gamma, st, fc, d,
          save_mask=psf_flag | _lib.RDXG_RESTORE_COBJ | _lib.RDXG_RESTORE_RESIDUAL, extras=extras)
    exe = _build(d)
    r = subprocess.run([exe, d], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    P = w.patches.cutouts.shape[0]
    alpha = np.fromfile(os.path.join(d, "alpha.out.f64")).reshape(P, job.n_images, job.n_modes)
    mets = np.fromfile(os.path.join(d, "metrics.out.f64")).reshape(P, st.max_metrics)
    rep = np.fromfile(os.path.join(d, "report.out.f64"))
    obj = np.fromfile(os.path.join(d, "objects.out.f32"), np.float32).reshape(
        P, job.n_objects, job.patch_size, job.patch_size)
    # the same solve through the Python harness (same library, same kernels, same inputs)
    s = S.Solver(job, max_patches=P)
    if extras:
        s.set_fit_plane(True)
        s.set_reg_alpha(extras["reg_alpha"])
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    if extras:
        s.set_initial_alpha(extras["init_alpha"])
    out = s.run(st)
    ref_obj = s.restore(out["alpha"], fc)
    np.testing.assert_array_equal(alpha, out["alpha"])
    for p in range(P):
        n = out["reports"][p].n_metrics
        assert rep[3 * p + 2] == n
        np.testing.assert_array_equal(mets[p, :n], out["metrics"][p, :n])
        assert rep[3 * p] == out["reports"][p].final_metric
        assert rep[3 * p + 1] == out["reports"][p].iterations
    np.testing.assert_allclose(obj, ref_obj, rtol=0, atol=1e-5 * np.abs(ref_obj).max())
    ps = job.patch_size
    ref = s.restore_outputs(out["alpha"], fc, psf="each" if cfg == "plain64" else "mean", cobj=True, residual=True)
    for name in ("psf", "cobj", "res"):
        key = "residual" if name == "res" else name
        got = np.fromfile(os.path.join(d, f"{name}.out.f32"), np.float32).reshape(ref[key].shape)
        scale = np.abs(ref["cobj"]).max() if name == "res" else np.abs(ref[key]).max()
        np.testing.assert_allclose(got, ref[key], rtol=0, atol=1e-5 * scale)
    # Solver::metric at the final alpha of the last patch
    m = s.metric(np.repeat(out["alpha"][P - 1:P], P, axis=0))[P - 1]
    assert abs(rep[3 * P] - m) <= 1e-6 * abs(m)
