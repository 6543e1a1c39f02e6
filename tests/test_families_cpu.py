"""Host logic of the family set: S-binning, root bounds, dedupe and the
reference's global bounds (no GPU)."""
import math
import pathlib
import re

import numpy as np

from cafe5_gb300.families import DEFAULT_BINS, FamilySet, bin_families, dedupe, global_bounds

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _set(rows):
    counts = np.asarray(rows, dtype=np.int32)
    return FamilySet([f"f{i}" for i in range(counts.shape[0])], counts)


def test_bin_widths_match_the_library():
    """The oracle is compared with the device at the library's bins, so the
    two lists must be the same."""
    src = (ROOT / "cafe5_gb300" / "csrc" / "cafe_abi.cu").read_text()
    m = re.search(r"kDefaultBins\[\]\s*=\s*\{([^}]*)\}", src)
    assert m, "kDefaultBins not found"
    assert tuple(int(x) for x in m.group(1).split(",")) == DEFAULT_BINS


def test_each_family_takes_the_smallest_bin_that_holds_its_states():
    rng = np.random.default_rng(3)
    mx = np.concatenate([np.arange(0, 900), rng.integers(0, 2000, 500)])
    fams = _set(np.stack([mx, mx // 2, np.zeros_like(mx)], axis=1))
    W, S, R = bin_families(fams)
    for m, w, s, r in zip(mx, W, S, R):
        need = math.ceil(1.2 * m) + 21            # states 0 .. ceil(1.2 m) + 20
        fits = [b for b in DEFAULT_BINS if b >= need]
        assert w == (fits[0] if fits else DEFAULT_BINS[-1])
        assert s == w - 1
        assert r == min(s, max(30, int(np.rint(1.25 * m))))
        assert r >= 1 and r <= s


def test_bin_cap_truncates_the_widest_families():
    fams = _set([[0, 1], [40, 3], [700, 2]])
    W, S, _ = bin_families(fams, cap=96)
    assert list(W) == [32, 96, 96]
    assert list(S) == [31, 95, 95]


def test_dedupe_refers_every_family_to_its_first_twin():
    rows = [[1, 2, 3], [0, 0, 0], [1, 2, 3], [4, 5, 6], [0, 0, 0], [1, 2, 3]]
    uniq, ref = dedupe(np.asarray(rows, dtype=np.int32))
    assert list(ref) == [0, 1, 0, 3, 1, 0]
    assert list(uniq) == [0, 1, 3]
    u0, r0 = dedupe(np.zeros((0, 3), dtype=np.int32))
    assert u0.size == 0 and r0.size == 0


def test_global_bounds_follow_the_reference_rule():
    # m = max(120, largest count); R = max(30, rint(1.25 m)), S = m + max(50, m / 5)
    # (integer division), as user_data sets them
    cases = {0: (170, 150), 7: (170, 150), 120: (170, 150), 121: (171, 151), 300: (360, 375), 1000: (1200, 1250)}
    for largest, want in cases.items():
        assert global_bounds(_set([[largest, 0], [1, 1]])) == want
    assert global_bounds(_set([[7, 0]]), floor=0) == (57, 30)
