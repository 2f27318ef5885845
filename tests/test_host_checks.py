"""Host-side argument checks that need no GPU."""
import numpy as np
import pytest

import paraht_gb300 as ph


def test_ht_rejects_non_triangular_b():
    rng = np.random.default_rng(0)
    A = rng.standard_normal((6, 6))
    B = rng.standard_normal((6, 6))  # general, not upper triangular
    with pytest.raises(ValueError, match="upper triangular"):
        ph.ht(A, B)


def test_ht_rejects_bad_shapes_and_precision():
    with pytest.raises(ValueError):
        ph.ht(np.zeros((3, 3)), np.zeros((4, 4)))
    with pytest.raises(ValueError):
        ph.ht(np.eye(3), np.eye(3), precision="fp32")
