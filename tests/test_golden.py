"""The oracle against the committed golden fixtures (tests/golden/*.npz,
made by tests/golden/make_golden.py): every output is reproduced bit for
bit, and the pair sets agree with an independent numpy brute force of the
reference's pair criterion (src/NeighborLists.jl:82-104: full list
d2 <= verlet^2, half list d2 < (rc*s_ij + skin)^2, minimum image
dx - round(dx/L)*L, src/MD.jl:115-117)."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def _golden_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_fixtures_present():
    names = {os.path.basename(p)[:-4] for p in FIXTURES}
    assert names == set(_golden_module().CASES)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_fixture(oracle, path):
    g = _golden_module()
    f = _load(path)
    p = g.params_from_json(str(f["params"]))
    noise = f["noise"] if f["noise"].size else None
    out = g.compute(p, f["r"], f["v"], f["D"], float(f["rc"]), noise)
    for k, v in out.items():
        assert np.array_equal(np.asarray(v), f[k]), k


def _brute_pairs(f, p):
    r, D = f["r"], f["D"]
    N, L = len(r), p.box_size
    rc, skin = float(f["rc"]), p.skin
    verlet = skin + rc * D.max()
    i, j = np.triu_indices(N, 1)
    d2 = np.zeros(len(i))
    for k in range(p.dims):
        dx = r[i, k] - r[j, k]
        dx = dx - np.rint(dx / L) * L
        d2 = d2 + dx * dx
    full = d2 <= verlet * verlet
    if p.potential == 0:
        s = np.full(len(i), p.lj_sigma * p.lj_sigma)
    else:
        s = (D[i] + D[j]) * 0.5 * (1.0 - p.b_zeta * np.abs(D[i] - D[j]))
    t = rc * s + skin
    half = full & (d2 < t * t)
    return np.stack([i[half], j[half]], 1), np.stack([i[full], j[full]], 1)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_pair_sets_match_brute_force(path):
    g = _golden_module()
    f = _load(path)
    p = g.params_from_json(str(f["params"]))
    half, full = _brute_pairs(f, p)
    assert np.array_equal(half, f["half_pairs"])
    assert np.array_equal(full, f["full_pairs"])
