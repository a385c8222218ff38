"""The oracle's restatement of the reference's analysis functions
(src/starrynight-analysis.c) against the reference's own outputs
(tests/golden/ref_analysis.npz): the potential and E-field maps bit for bit,
the order parameters and the correlation histogram to the reference's float
accumulation."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_analysis.npz"))
CASES = sorted({k.split("/")[0] for k in GOLD.files})


def _case(name):
    lat = GOLD[name + "/lattice"]
    shape = tuple(int(v) for v in GOLD[name + "/shape"])
    return lat, shape


@pytest.mark.parametrize("name", CASES)
def test_potential_map_bitwise(name):
    lat, shape = _case(name)
    pot = O.potential_map(lat[:, 0], lat[:, 1], lat[:, 2], lat[:, 3], shape, 6)
    assert np.array_equal(pot, GOLD[name + "/potential"])


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("cutoff,half,key", [(4, False, "efield4"), (2, True, "efieldoffset2")])
def test_efield_map_bitwise(name, cutoff, half, key):
    lat, shape = _case(name)
    ef = O.efield_map(lat[:, 0], lat[:, 1], lat[:, 2], shape, cutoff, half)
    assert np.array_equal(ef, GOLD[name + "/" + key])


@pytest.mark.parametrize("name", CASES)
def test_order_parameters(name):
    lat, _ = _case(name)
    pol, landau, s3 = O.order_params(lat[:, 0], lat[:, 1], lat[:, 2])
    ref_pol, ref_landau = GOLD[name + "/order"]
    # polarisation(): double sum of the x components in both
    assert pol == pytest.approx(ref_pol, rel=1e-12, abs=1e-15)
    # landau_order(): the reference sums the orientation in float
    assert landau == pytest.approx(ref_landau, rel=1e-5, abs=1e-3)
    assert landau == pytest.approx(float(np.dot(s3, s3)), rel=1e-14)


@pytest.mark.parametrize("name", CASES)
def test_radial_order(name):
    lat, shape = _case(name)
    rows = GOLD[name + "/rdf"]  # r^2, r, <FE>, <AFE>, count, T for bins < 81 with count > 0
    bins = rows[:, 0].astype(int)
    # the reference's own float histogram reproduces its printed means exactly
    fe, afe, cnt = O.radial_order(lat[:, 0], lat[:, 1], lat[:, 2], shape, 9, float_sums=True)
    assert list(bins) == [b for b in range(81) if cnt[b] > 0]
    assert np.array_equal(rows[:, 4].astype(np.int64), cnt[bins])
    c32 = cnt[bins].astype(np.float32)
    for col, sums in ((2, fe), (3, afe)):
        mine = ["%f" % v for v in sums[bins].astype(np.float32) / c32]
        ref = ["%f" % v for v in rows[:, col]]
        assert mine == ref
    # the FP64 sums (what the GPU reports) differ from the float ones only by the float rounding
    fe64, afe64, cnt64 = O.radial_order(lat[:, 0], lat[:, 1], lat[:, 2], shape, 9)
    assert np.array_equal(cnt64, cnt)
    tol = 1e-6 + cnt[bins] * 2.0 ** -24  # float accumulation bound over count terms of magnitude <= 1
    assert np.all(np.abs(fe64[bins] / cnt[bins] - rows[:, 2]) <= tol)
    assert np.all(np.abs(afe64[bins] / cnt[bins] - rows[:, 3]) <= 3 * tol)
