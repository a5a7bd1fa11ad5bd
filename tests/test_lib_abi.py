"""The C-ABI library loads on a host without a GPU and exports every declared symbol."""
import os
import re

from redux_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "rdxg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set(re.findall(r"^\s*(?:int|int32_t|int64_t|const char\*)\s+(rdxg_\w+)\s*\(", src, flags=re.M))
    return names


def test_header_declares_the_python_table():
    assert declared_functions() == set(_lib.EXPORTED)


def test_library_exports_every_symbol():
    L = _lib.load()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.rdxg_version() >= 100


def test_unsupported_size_is_rejected_before_any_device_call():
    """An OTF size without compiled kernels: rdxg_create answers RDXG_ERR_UNSUPPORTED with a
    message, before it touches a device (so this runs on a host without a GPU)."""
    import pytest
    from redux_gb300 import solver as S, synth
    job = synth.make_job(96, 8, synth.LAYOUT_1OBJ(2))
    with pytest.raises(S.SolverError, match=r"status 2: otf_size not compiled"):
        S.Solver(job, max_patches=1, precision="fp64")


def test_eval_chunk_out_of_range_is_rejected_before_any_device_call():
    """rdxg_geometry.eval_chunk takes 0 (the default, 6) to 32 images per work item."""
    import pytest
    from redux_gb300 import solver as S
    from tests.conftest import workload
    w = workload("production88", n_patches=2, frames=4)
    for bad in (-1, 33):
        with pytest.raises(S.SolverError, match=r"eval_chunk must be 0\.\.32"):
            S.Solver(w.job, max_patches=1, eval_chunk=bad)
