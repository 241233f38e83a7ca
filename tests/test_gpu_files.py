"""The file API of the GPU library against the CPU oracle (GPU).

Every field, force, map, object and stress file written by the GPU library
(FP64 populations) must be byte-identical to the oracle's, whose files are
themselves byte-identical to the strict reference build's (test_oracle.py,
tests/golden/files.json).  Lattices reloaded from those files (lbloadvel
binary and ascii, lbloadobj) must equal the oracle's bit for bit, and so
must a tracer set by mpsubs and advanced on a live flow.

Reference routines: lbsavevel / lbloadvel src/lbstore.c:227-404, lbsavestr
:412-515, lbsaveobj / lbloadobj :523-586, lbsavefrc :595-640, lbsavemap
:647-678, vgrab / vsave src/lbmeasure.c:129-203, mpsubs src/mpobjs.c:188-226.
"""

import numpy as np
import pytest

import scenarios as S
from golden.make_golden import FILE_CASES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", sorted(FILE_CASES))
def test_files_byte_identical(gpu, orc, tmp_path, case):
    cfg = FILE_CASES[case]
    (tmp_path / "g").mkdir()
    (tmp_path / "o").mkdir()
    lg, fg = S.file_case(gpu, str(tmp_path / "g"), **cfg)
    lo, fo = S.file_case(orc, str(tmp_path / "o"), **cfg)
    assert fg.keys() == fo.keys()
    differ = [k for k in fg if fg[k] != fo[k]]
    assert not differ, differ
    # lbsavestr advanced both lattices one step: still bit-equal
    assert lg.step == lo.step
    assert np.array_equal(lg.pops(), lo.pops())
    for kind in ("vel.bin", "vel.txt"):
        _, pg = S.reload_case(gpu, str(tmp_path / "g"), kind, **cfg)
        _, po = S.reload_case(orc, str(tmp_path / "o"), kind, **cfg)
        assert np.array_equal(pg, po), (kind, np.abs(pg - po).max())
    _, og = S.reload_case(gpu, str(tmp_path / "g"), "obj.txt", **cfg)
    _, oo = S.reload_case(orc, str(tmp_path / "o"), "obj.txt", **cfg)
    assert np.array_equal(og, oo)


def test_mpsubs_bit_exact(gpu, orc, tmp_path):
    g0, g1 = S.mpsubs_case(gpu, str(tmp_path))
    o0, o1 = S.mpsubs_case(orc, str(tmp_path))
    assert np.array_equal(g0, o0)
    assert np.count_nonzero(g0) > 0
    assert np.array_equal(g1, o1), np.abs(g1 - o1).max()
