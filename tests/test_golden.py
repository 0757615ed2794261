"""The oracle against the committed golden fixtures (tests/golden/*.npz, made by
tests/golden/make_golden.py): index maps bit-exact, values within 1e-12 relative L2 (the
oracle's threaded sums may round differently from run to run), iteration counts equal."""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import make_golden as G  # noqa: E402

INDEX_KEYS = {"dof_map", "vector_dof_map", "cmap", "iterations", "cells", "cell_dofs", "hang_count", "hang_master",
              "hang_weight"}


@pytest.mark.parametrize("name", sorted(G.FIXTURES))
def test_oracle_reproduces_golden(name):
    ref = np.load(GOLDEN / f"{name}.npz")
    got = G.FIXTURES[name]()
    assert set(got) == set(ref.files)
    for k in ref.files:
        if k in INDEX_KEYS:
            assert np.array_equal(np.asarray(got[k]), ref[k]), k
        elif k == "residual":
            assert float(got[k]) < 1e-11
        else:
            a, b = np.asarray(got[k]), ref[k]
            assert np.linalg.norm(a - b) <= 1e-12 * max(np.linalg.norm(b), 1e-300), k
