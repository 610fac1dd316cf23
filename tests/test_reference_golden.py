"""The oracle against outputs of the reference's own device code.

tests/golden/reference_pairs.npz was produced by oracle/ref_harness/run_ref.py,
which runs the reference's points_to_rays / hit / em_wave (compiled from its
sources by oracle/ref_harness/build_ref.py, default and --fmad=false builds) on
two seeded scenes: the 8x8-array direct scene (64 x 2,664 pairs, 1,024
triangles, reference pair rule) and a random scene (40 x 500 pairs, 300 large
triangles, all pairs tested, alpha = 0.05)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_pairs.npz")


def _case(d, k):
    return {x: d[f"{k}_{x}"] for x in ("src", "snk", "snk_n", "verts", "faces", "E", "alpha", "beta", "flag",
                                       "sample")}


@pytest.mark.parametrize("case", ["direct", "random"])
@pytest.mark.parametrize("variant", ["fma", "nofma"])
def test_oracle_masks_equal_reference_masks(case, variant):
    d = np.load(GOLD)
    c = _case(d, case)
    N, M = c["src"].shape[0], c["snk"].shape[0]
    ref = np.unpackbits(d[f"{case}_{variant}_vis"])[:N * M].reshape(N, M).astype(bool)
    om = O.mask_brute(c["src"], c["snk"], O.pack_triangles(c["verts"], c["faces"]), self_to_self=bool(c["flag"]))
    assert np.array_equal(om, ref), f"{int((om != ref).sum())} of {om.size} pairs differ"
    assert 0 < om.sum() < om.size


@pytest.mark.parametrize("case", ["direct", "random"])
def test_oracle_fields_match_reference_to_its_fp32_phase(case):
    """The reference forms beta*r in FP32 (lyceanem/src/em.cuh:80): its phase error grows with beta*r,
    about 3e-4 rad at beta*r ~ 2,100 (direct scene), so its field agrees with the FP64 oracle to 1e-3."""
    d = np.load(GOLD)
    c = _case(d, case)
    om = O.mask_brute(c["src"], c["snk"], O.pack_triangles(c["verts"], c["faces"]), self_to_self=bool(c["flag"]))
    S = O.pair_field(c["src"], c["E"], c["snk"], c["snk_n"], om, float(c["alpha"]), float(c["beta"])).reshape(-1, 3)
    ref = S[c["sample"]]
    for variant in ("fma", "nofma"):
        got = d[f"{case}_{variant}_field"].astype(np.float32).view(np.complex64).reshape(-1, 3)
        assert np.all((np.abs(got) > 0) == (np.abs(ref) > 0))
        assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-3
