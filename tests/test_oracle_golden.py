"""The oracle reproduces every golden fixture made by the reference itself."""

import numpy as np
import pytest

import cases


@pytest.mark.parametrize("name", cases.CASES)
def test_oracle_matches_reference_fixture(name):
    arrays, _ = cases.golden()
    got = cases.oracle_case(name)
    assert got.shape == arrays[name].shape
    assert cases.rel_l2(got, arrays[name]) < 1e-12


def test_fixtures_are_nontrivial():
    arrays, _ = cases.golden()
    for name in cases.CASES:
        assert np.all(np.isfinite(arrays[name])), name
        assert np.linalg.norm(arrays[name]) > 0, name
    # distinct frames really move
    fr = arrays["atm_frames"]
    assert np.linalg.norm(fr[1] - fr[0]) > 1e-3 * np.linalg.norm(fr[0])


def test_oracle_compaction_keeps_stencil_and_window():
    import oracle

    buf = np.arange(20.0)[:, None] * np.ones((1, 3))
    base, fill = oracle.compact_row_ring(buf, 100, 20, 2, 112.7)
    # keeps rows from floor(112.7) - 1 = 111 on
    assert base == 111 and fill == 9
    assert buf[0, 0] == 11.0
    # a readable row far ahead is capped by the stencil rows
    buf = np.arange(20.0)[:, None] * np.ones((1, 3))
    base, fill = oracle.compact_row_ring(buf, 0, 20, 2, 1e6)
    assert (base, fill) == (18, 2)
