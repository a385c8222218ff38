"""Self-consistency of the FP64 oracle: site-energy differences equal total
energy differences, the analytic gradient equals finite differences, and
the colour-sweep mirror's bookkeeping matches full recomputes."""
import numpy as np
import pytest

from oracle import oracle as O


def _random_lattice(n, rng, vac=0.0):
    v = rng.normal(size=(n, 3))
    v = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    ln = np.ones(n, np.float32)
    if vac:
        ln[rng.random(n) < vac] = 0.0
        v[ln == 0] = 0.0
    return [np.ascontiguousarray(v[:, k]) for k in range(3)], ln


@pytest.mark.parametrize("shape,rc,K", [((6, 6, 6), 2, 0.0), ((8, 6, 10), 3, 0.3), ((10, 10, 1), 3, 0.0)])
def test_delta_energy_equals_total_difference(shape, rc, K):
    rng = np.random.default_rng(1)
    X, Y, Z = shape
    m = O.make_model(X, Y, Z, rc, T=300.0, efield=(0.1, -0.05, 0.2), K=K, cage_strain=0.8)
    (px, py, pz), ln = _random_lattice(X * Y * Z, rng, vac=0.2)
    E0 = O.energy64(m, px, py, pz, ln)["E"]
    for _ in range(10):
        i = int(rng.integers(X * Y * Z))
        if ln[i] == 0:
            continue
        v = rng.normal(size=3)
        v = (v / np.linalg.norm(v)).astype(np.float32)
        dE = O.delta_energy64(m, px, py, pz, ln, i, v)
        old = (px[i], py[i], pz[i])
        px[i], py[i], pz[i] = v
        E1 = O.energy64(m, px, py, pz, ln)["E"]
        assert abs((E1 - E0) - dE) < 1e-9 * max(1.0, abs(E0))
        px[i], py[i], pz[i] = old


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(2)
    X, Y, Z = 6, 6, 6
    m = O.make_model(X, Y, Z, 3, T=300.0, efield=(0.05, 0.0, 0.05), cage_strain=0.5)
    (px, py, pz), ln = _random_lattice(X * Y * Z, rng, vac=0.1)
    r = O.energy64(m, px, py, pz, ln, grad=True)
    g = r["grad"]
    h = 1e-3  # float32 lattice: central differences on the float grid are exact for a quadratic form
    for i in rng.choice(np.nonzero(ln)[0], 8, replace=False):
        for k, arr in enumerate((px, py, pz)):
            o = arr[i]
            arr[i] = o + np.float32(h)
            ep = O.energy64(m, px, py, pz, ln)["E"]
            hp = float(arr[i]) - float(o)
            arr[i] = o - np.float32(h)
            em = O.energy64(m, px, py, pz, ln)["E"]
            hm = float(o) - float(arr[i])
            arr[i] = o
            fd = (ep - em) / (hp + hm)
            assert abs(fd - g[i, k]) < 1e-6 * max(1.0, abs(g[i, k]))


def test_colour_sweep_bookkeeping():
    import starrynight_gb300 as sn
    rng = np.random.default_rng(3)
    X = Y = Z = 8
    m = O.make_model(X, Y, Z, 3, T=300.0, efield=(0, 0, 0.1))
    (px, py, pz), ln = _random_lattice(X * Y * Z, rng, vac=0.3)
    st = O.make_stream(11, 1.0, 1.0)
    sched = O.make_schedule(sn.plan_schedule(X, Y, Z, 3))
    E0 = O.energy64(m, px, py, pz, ln)["E"]
    tot = 0.0
    for s in range(3):
        r = O.colour_sweep(m, sched, st, s, px, py, pz, ln)
        tot += r.dE_sum
        assert 0 < r.accepted < int((ln > 0).sum())
    E1 = O.energy64(m, px, py, pz, ln)["E"]
    assert abs((E1 - E0) - tot) < 1e-9 * abs(E0)
    assert np.allclose(px[ln == 0], 0) and np.allclose(np.sqrt(px ** 2 + py ** 2 + pz ** 2)[ln > 0], 1, atol=1e-6)
