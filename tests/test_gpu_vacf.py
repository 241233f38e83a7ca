"""Tracer velocity autocorrelation (reference src/mpvacf.c) on the GPU
library against the CPU oracle, which equals the reference build bit for
bit (test_oracle.py).  The initialisations run on the host mirrors in the
reference's order; each mpvacf call runs on the GPU, whose sums are
ordered differently, so the diffusion coefficient and the fields are
compared to 1e-10 relative (FP64 populations and tracers); the written
file to its printed digits."""

import numpy as np
import pytest

import scenarios as S
from test_oracle import VACF_CASES

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.mark.parametrize("n", range(len(VACF_CASES)))
def test_vacf_matches_oracle(gpu, orc, tmp_path, n):
    kw = VACF_CASES[n]
    (tmp_path / "g").mkdir()
    (tmp_path / "o").mkdir()
    dg, pg, p2g, fg = S.vacf_case(gpu, str(tmp_path / "g"), **kw)
    do, po, p2o, fo = S.vacf_case(orc, str(tmp_path / "o"), **kw)
    assert abs(dg - do) <= TOL * abs(do), (dg, do)
    assert np.abs(pg - po).max() <= TOL * np.abs(po).max()
    assert np.abs(p2g - p2o).max() <= TOL * np.abs(p2o).max()
    lg, lo = fg.decode().split("\n"), fo.decode().split("\n")
    assert len(lg) == len(lo)
    for a, b in zip(lg, lo):
        if a:
            va, vb = [float(v) for v in a.split()], [float(v) for v in b.split()]
            assert va[0] == vb[0]
            assert all(abs(x - y) <= 1e-5 * max(abs(y), 1e-30) for x, y in zip(va[1:], vb[1:])), (a, b)
