"""CPU emulation (numpy float32) of the split-precision pair arithmetic of
k_force.cu against the oracle's FP64 pair forces, on a relaxed soft-sphere
start (capped steepest descent from random positions: pairs near contact
whose forces partly cancel -- the hardest state for FP32 pair arithmetic).

Two forms are emulated operation by operation (FMA as one rounding):
  * the kept form: positions in 32-bit fixed point of the box, the pair
    difference and r^2 exact in integers, the pair diameter s^2 and the
    ratio x = r^2 / s^2 with their rounding errors carried (error-free sum,
    FMA residuals, first order);
  * the plain FP32 form: FP32 offsets from a power-of-two grid, s^2 and x
    in plain FP32.
The kept form must meet the 1e-5 force bar with margin and be well below
the plain form; the per-particle sum order is not what limits the error
(FP32 and FP64 sums of the same FP32 pair forces agree to a few percent).
"""
import numpy as np
import pytest

f32 = np.float32


def _fma(a, b, c):
    """float32 fused multiply-add: the exact product of two float32 fits a
    float64, one rounding to float32 after the add"""
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(np.float32)


def _system(oracle, N=4096, seed=3):
    from oracle import pyoracle as O
    from simulationcode_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    s = W.berthier_spec(N, 3, 0, rng, dt=0.005)
    p = O.make_params(3, O.POT_BERTHIER, O.NEWTONIAN, N, s.box_size, s.force_cutoff2, 0.3)
    o = O.OracleSystem(p, s.r, s.D, force_cutoff=1.25, maxK=200)
    o.relax_capped(300, 1e-3, 0.05)
    o.update_neighbor_lists()
    F64 = o.pair_forces()
    I = np.repeat(np.arange(N), o.nn_full)
    J = o.list_full[np.arange(o.list_full.shape[1])[None, :] < o.nn_full[:, None]]
    return o, p, F64, I, J


def _kept_form(o, p, I, J):
    L = p.box_size
    c2, c4 = f32(p.b_c2), f32(p.b_c4)
    X = np.mod(np.round(o.r / L * 2.0 ** 32), 2.0 ** 32).astype(np.uint64).astype(np.uint32)
    d = X[I].astype(np.int64) - X[J].astype(np.int64)
    d = ((d + 2 ** 31) % 2 ** 32 - 2 ** 31).astype(np.int64)          # int32 wraparound
    u = np.float32(L / 2.0 ** 32)
    r2 = ((d ** 2).sum(1).astype(np.float64).astype(np.float32) * f32(u * u)).astype(np.float32)
    dx = (d.astype(np.float32) * u).astype(np.float32)
    D = o.D.astype(np.float32)
    Di, Dj = D[I], D[J]
    zeta = f32(p.b_zeta)
    zlo = f32(p.b_zeta - np.float64(zeta))
    a, b = np.maximum(Di, Dj), np.minimum(Di, Dj)
    S = a + b
    eS = b - (S - a)
    dd = a - b
    pz = zeta * dd
    ep = _fma(zeta, dd, -pz) + zlo * dd
    T = f32(1) - pz
    eT = ((f32(1) - T) - pz) - ep
    m = S * T
    em = _fma(S, T, -m) + (S * eT + eS * T)
    m, em = m * f32(0.5), em * f32(0.5)
    q = m * m
    eq = _fma(m, m, -q) + f32(2) * m * em
    inv = f32(1) / q
    x = r2 * inv
    x = _fma(_fma(-x, q, r2) - x * eq, inv, x)
    xsq = x * x
    xi14 = f32(1) / (xsq * xsq * xsq * x)
    B = _fma(f32(-6), xi14, _fma(f32(2) * c4, x, c2))
    F0 = f32(-2) * inv * B
    Fr = np.where(r2 <= f32(1.5625) * q, _fma(-F0, eq * inv, F0), f32(0))
    return Fr[:, None] * dx


def _plain_form(o, p, I, J):
    L = p.box_size
    h = 0.5
    while L / h > 1022:
        h *= 2
    g = np.round(o.r / h) * h
    of, gf = (o.r - g).astype(np.float32), g.astype(np.float32)
    aa = of[I] - of[J]
    G0 = gf[I] - gf[J]
    dx0 = aa + G0
    half = f32(L / 2)
    sg = np.where(dx0 > half, f32(1), np.where(dx0 < -half, f32(-1), f32(0)))
    Lhi = f32(np.floor(L / h) * h)
    Llo = f32(L - np.floor(L / h) * h)
    dx = np.where(sg == 0, dx0, (aa - sg * Llo) + (G0 - sg * Lhi)).astype(np.float32)
    r2 = _fma(dx[:, 0], dx[:, 0], _fma(dx[:, 1], dx[:, 1], dx[:, 2] * dx[:, 2]))
    D = o.D.astype(np.float32)
    Di, Dj = D[I], D[J]
    md = (Di + Dj) * f32(0.5) * (f32(1) - f32(p.b_zeta) * np.abs(Di - Dj))
    mds = md * md
    inv = f32(1) / mds
    ix2 = r2 * inv
    ix4 = ix2 * ix2
    xi14 = f32(1) / (ix4 * ix4 * ix4 * ix2)
    B = f32(p.b_c2) + f32(2) * f32(p.b_c4) * ix2 - f32(6) * xi14
    Fr = np.where(r2 <= f32(1.5625) * mds, f32(-2) * inv * B, f32(0))
    return Fr[:, None] * dx


def _rel(F, F64):
    return float(np.sqrt(((F - F64) ** 2).sum() / (F64 ** 2).sum()))


def test_kept_split_form_meets_the_force_bar_at_a_quench(oracle):
    o, p, F64, I, J = _system(oracle)
    N = p.N
    res = {}
    for name, form in (("kept", _kept_form), ("plain", _plain_form)):
        fp = form(o, p, I, J)
        F32 = np.zeros((N, 3), np.float32)
        np.add.at(F32, I, fp)                       # FP32 per-particle sums in list order
        Fex = np.zeros((N, 3))
        np.add.at(Fex, I, fp.astype(np.float64))    # the same pair forces summed in FP64
        res[name] = (_rel(F32.astype(np.float64), F64), _rel(Fex, F64))
    print("force relative RMS (FP32 sum, FP64 sum):", res)
    kept, plain = res["kept"], res["plain"]
    assert kept[0] <= 8e-6
    assert kept[0] <= 0.7 * plain[0]
    assert kept[1] == pytest.approx(kept[0], rel=0.05) and plain[1] == pytest.approx(plain[0], rel=0.05)
