"""The oracle against its committed golden vectors (tests/golden/make_golden.py): a change to
the FP64 restatement, which every GPU test compares against, fails here on the CPU."""
import os

import numpy as np

from tests.golden import make_golden as G

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_reproduces_its_golden_vectors():
    ref = np.load(os.path.join(HERE, "golden", "oracle_golden.npz"))
    got = {}
    for name, w in G.cases():
        got.update(G.compute(name, w))
    assert set(got) == set(ref.files)
    for k in ref.files:
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-9, atol=1e-12 * np.abs(ref[k]).max(), err_msg=k)
