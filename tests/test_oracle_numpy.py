"""The oracle against a second, independent restatement of the reference's
pair expressions: numpy over all pairs (minimum image by round-half-even, as
Julia's round), no neighbour list, no cell list, no shared code with the C
oracle.  Each expression follows the reference line it cites:

  * soft spheres ("Berthier") force over r: src/MD.jl:116-128 (3D) and the
    2D loop of the same form, src/MD.jl:194-238;
  * soft-sphere energy: berthier_inner_loop3/2,
    src/AuxiliaryFunctions.jl:381-444;
  * LJ 3D force over r: compute_forces_lj_3d, src/MD.jl:140-191;
  * LJ 3D energy: LJ_inner_loop, src/AuxiliaryFunctions.jl:477-507;
  * LJ 2D force and energy: the generic loops, src/MD.jl:291-309 and
    src/AuxiliaryFunctions.jl:571-581 (find_mean_D(LJ) = sigma^2, squared);
  * energy = half the sum over ordered pairs (calculate_full_energy,
    src/AuxiliaryFunctions.jl:22-34); virial = sum over pairs of
    (F/r) r^2 (the build's definition).

and the time step written out the same way (Newtonian / Langevin velocity
Verlet with the centre-of-mass removal, src/MD.jl:499-542; Brownian as
intended by src/MD.jl:429-471), 10 steps beside the oracle's with the same
noise; the inherent-structure descent (src/InherentStructure.jl:5-56),
200 iterations; and swap Monte Carlo sweeps (src/MC.jl:21-156) with the
oracle's keyed draws.

Tolerance: forces max|dF| <= 1e-12 max|F|; energy and virial relative
1e-12 (the two differ only in summation order); positions and velocities
after 10 steps within 1e-11.
"""
import numpy as np
import pytest

from cases import make_case


def _pair_terms(p, r, D):
    """(F/r, V, dx) for every ordered pair i != j, from the reference's
    expressions"""
    N, dims, L = p.N, p.dims, p.box_size
    dx = r[:, None, :] - r[None, :, :]
    dx -= np.round(dx / L) * L                       # src/MD.jl:116-118
    r2 = (dx * dx).sum(-1)
    np.fill_diagonal(r2, np.inf)
    rc2 = p.force_cutoff2
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        if p.potential == 1:  # Berthier
            Di, Dj = D[:, None], D[None, :]
            mean_d = (Di + Dj) * 0.5 * (1.0 - p.b_zeta * np.abs(Di - Dj))
            s2 = mean_d * mean_d
            inv = 1.0 / s2
            x = r2 * inv
            x4 = x * x
            xi14 = 1.0 / (x4 * x4 * x4 * x)
            out = rc2 * s2 < r2
            Fr = np.where(out, 0.0, -2.0 * inv * (p.b_c2 + 2.0 * p.b_c4 * x - 6.0 * xi14))
            ix2 = r2 / s2
            ix4 = ix2 * ix2
            xi12 = 1.0 / (ix4 * ix4 * ix4)
            V = np.where(out, 0.0, xi12 + p.b_c4 * ix4 + p.b_c2 * ix2 + p.b_c0)
        elif dims == 2:  # LJ 2D: the generic loop, src/MD.jl:291-309, and find_energy's
            # generic branch, src/AuxiliaryFunctions.jl:571-581; find_mean_D(LJ) = sigma^2
            # (src/InteractionPotential.jl:5-7), squared again; strict '>' cut
            mds = (p.lj_sigma ** 2) * (p.lj_sigma ** 2)
            inside = rc2 * mds > r2
            inv = 1.0 / r2
            xi2 = mds * inv
            xi6 = xi2 * xi2 * xi2
            xi12 = xi6 * xi6
            Fr = np.where(inside, p.lj_eps * (48.0 * xi12 - 24.0 * xi6) * inv, 0.0)
            y2 = mds / r2
            y4 = y2 * y2
            y6 = y2 * y4
            y12 = y6 * y6
            V = np.where(inside, 4.0 * p.lj_eps * (y12 - y6) - p.lj_Uc, 0.0)
        else:  # LJ, 3D
            s2 = p.lj_sigma * p.lj_sigma
            xi2 = s2 / r2
            xi6 = xi2 * xi2 * xi2
            xi12 = xi6 * xi6
            Fr = np.where(rc2 < r2, 0.0, p.lj_eps * (48.0 * xi12 - 24.0 * xi6) / r2)
            V = np.where(rc2 * s2 < r2, 0.0, 4.0 * p.lj_eps * (xi12 - xi6) - p.lj_Uc)
    np.fill_diagonal(Fr, 0.0)
    np.fill_diagonal(V, 0.0)
    return Fr, V, dx, np.where(np.isfinite(r2), r2, 0.0)


@pytest.mark.parametrize("pot,dims,N", [(1, 3, 343), (1, 2, 400), (0, 3, 343), (0, 2, 400)])
def test_oracle_matches_numpy_restatement(oracle, pot, dims, N):
    p, r, v, D, rc = make_case(pot, dims, oracle.NEWTONIAN, N, seed=9, mc_sweeps=10)
    s = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    s.update_neighbor_lists()
    F_orc = s.pair_forces()
    Fr, V, dx, r2 = _pair_terms(p, np.asarray(r, float), np.asarray(D, float))
    F_np = (Fr[:, :, None] * dx).sum(1)
    assert np.abs(F_orc - F_np).max() <= 1e-12 * np.abs(F_np).max()
    assert s.full_energy() == pytest.approx(V.sum() / 2.0, rel=1e-12)
    assert s.virial() == pytest.approx((Fr * r2).sum() / 2.0, rel=1e-12)
    assert np.abs(F_np).max() > 1.0 and (Fr != 0).sum() > N  # the case exercises the potential


def _forces(p, r, D):
    Fr, V, dx, r2 = _pair_terms(p, r, D)
    return (Fr[:, :, None] * dx).sum(1)


def _numpy_step(p, r, v, F, D, xi):
    """one do_time_step of the reference written out in numpy: Newtonian /
    Langevin src/MD.jl:499-542 (add_new_random_force! :30-45), Brownian as
    intended by src/MD.jl:429-471 (forces + noise :62-74, the mean force
    removed, r += (dt/gamma) F, wrapped).  Returns (r, v, F)."""
    L, dt, m = p.box_size, p.dt, p.m
    if p.dynamics == 2:  # Brownian
        F = _forces(p, r, D) + np.sqrt(2 * p.kBT * p.gamma / dt) * xi
        F = F - F.sum(0) / p.N
        rn = r + (dt / p.gamma) * F
        rn -= np.floor(rn / L) * L
        return rn, v, F
    v = v + dt * F / (2.0 * m)
    rn = r + dt * v
    rn -= np.floor(rn / L) * L
    F = _forces(p, rn, D)
    if p.dynamics == 1:  # Langevin
        F = F + (-p.gamma * v + np.sqrt(2 * p.kBT * p.gamma / dt) * xi)
    v = v + dt * F / (2.0 * m)
    v = v - v.sum(0) / p.N
    return rn, v, F


@pytest.mark.parametrize("pot,dims,dyn", [(1, 3, 0), (0, 3, 1), (1, 2, 1), (1, 3, 2), (1, 2, 2)])
def test_oracle_time_step_matches_numpy_restatement(oracle, pot, dims, dyn):
    N, nsteps = (343 if dims == 3 else 400), 10
    dt = 2e-5 if dyn == 2 else 0.005
    p, r, v, D, rc = make_case(pot, dims, dyn, N, seed=13, dt=dt)
    s = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    s.update_neighbor_lists()
    s.calculate_new_forces(np.zeros((N, dims)))
    rn, vn, Fn = s.r.copy(), s.v.copy(), s.F.copy()
    noise = np.random.default_rng(17).standard_normal((nsteps, N, dims))
    for k in range(nsteps):
        s.step(noise[k] if dyn else None)
        rn, vn, Fn = _numpy_step(p, rn, vn, Fn, np.asarray(D, float), noise[k])
    d = s.r - rn
    d -= np.round(d / p.box_size) * p.box_size
    assert np.abs(d).max() <= 1e-11
    if dyn != 2:
        assert np.abs(s.v - vn).max() <= 1e-11 * max(1.0, np.abs(vn).max())


@pytest.mark.parametrize("pot,dims,N,dt", [(1, 3, 216, 0.005), (1, 2, 256, 1e-3), (0, 3, 216, 1e-3)])
def test_oracle_minimiser_matches_numpy_restatement(oracle, pot, dims, N, dt):
    """find_inherent_structure (src/InherentStructure.jl:5-56) written out in
    numpy: v = F dt, capped so that max |v| <= max_step_size, r += v
    wrapped; 200 iterations of it beside the oracle's stopped at
    max_iterations = 200"""
    p, r, v, D, rc = make_case(pot, dims, 0, N, seed=21)
    s = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    st, it = oracle.find_inherent_structure(s, tolerance=1e-12, max_iterations=200, max_step_size=0.001, dt=dt)
    assert st == 2  # stopped by max_iterations, after exactly 200 iterations
    rn, L, Dn = np.array(r, float), p.box_size, np.asarray(D, float)
    for _ in range(200):
        step = _forces(p, rn, Dn) * dt
        size = np.sqrt((step * step).sum(1)).max()
        if size > 0.001:
            step *= 0.001 / size
        rn = rn + step
        rn -= np.floor(rn / L) * L
    d = s.r - rn
    d -= np.round(d / L) * L
    assert np.abs(d).max() <= 1e-10


def _particle_energy(p, i, ri, Di, r, D):
    """find_energy (src/AuxiliaryFunctions.jl:546-584, berthier_inner_loop3/2)
    over all other particles"""
    d = ri[None, :] - r
    d -= np.round(d / p.box_size) * p.box_size
    r2 = (d * d).sum(1)
    r2[i] = np.inf
    mean_d = (Di + D) * 0.5 * (1.0 - p.b_zeta * np.abs(Di - D))
    s2 = mean_d * mean_d
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        ix2 = r2 / s2
        ix4 = ix2 * ix2
        xi12 = 1.0 / (ix4 * ix4 * ix4)
        V = np.where(p.force_cutoff2 * s2 < r2, 0.0, xi12 + p.b_c4 * ix4 + p.b_c2 * ix2 + p.b_c0)
    return V.sum()


@pytest.mark.parametrize("dims,N", [(3, 216), (2, 256)])
def test_oracle_mc_matches_numpy_restatement(oracle, dims, N):
    """do_MC_step! (src/MC.jl:139-156) with do_translation_step! (:21-47) and
    do_swap_step! (:67-110) written out in numpy over all pairs, with the
    oracle's keyed draws (u[0] move kind, u[1] acceptance, u[2..] the
    displacement, u[5] the swap partner, drawn uniformly: the evident intent
    of src/MC.jl:152, whose ceil(rand()/N) always gives particle 1): the
    same moves accepted, the same positions and diameters, the same summed
    dE"""
    p, r, v, D, rc = make_case(1, dims, 0, N, seed=4, skin=0.6)
    p.kBT = 0.5
    s = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    s.update_neighbor_lists()
    nsweeps, max_disp, swap_prob, seed = 3, 0.08, 0.3, 77
    counts, de = s.mc_sweeps(nsweeps, max_disp, swap_prob, seed)
    rn, Dn, L = np.array(r, float), np.array(D, float), p.box_size
    cn, den = np.zeros(4, np.int64), 0.0
    for sw in range(nsweeps):
        for i in range(N):
            u = oracle.mc_uniforms(seed, sw, i)
            if u[0] > swap_prob:  # translation
                dr = u[2:2 + dims] * 2.0 * max_disp - max_disp
                e_old = _particle_energy(p, i, rn[i], Dn[i], rn, Dn)
                rnew = rn[i] + dr
                rnew -= np.floor(rnew / L) * L
                dE = _particle_energy(p, i, rnew, Dn[i], rn, Dn) - e_old
                cn[1] += 1
                if min(1.0, np.exp(-dE / p.kBT)) > u[1]:
                    cn[0] += 1
                    rn[i] = rnew
                    den += dE
            else:  # swap
                j = min(int(u[5] * N), N - 1)
                if j == i or abs(Dn[i] - Dn[j]) > 0.2:
                    continue
                Di, Dj = Dn[i], Dn[j]
                old = _particle_energy(p, i, rn[i], Di, rn, Dn) + _particle_energy(p, j, rn[j], Dj, rn, Dn)
                Dn[i], Dn[j] = Dj, Di
                new = _particle_energy(p, i, rn[i], Dj, rn, Dn) + _particle_energy(p, j, rn[j], Di, rn, Dn)
                dE = new - old
                cn[3] += 1
                if min(1.0, np.exp(-dE / p.kBT)) > u[1]:
                    cn[2] += 1
                    den += dE
                else:
                    Dn[i], Dn[j] = Di, Dj
    assert np.array_equal(counts, cn) and cn[0] > 0 and cn[2] > 0
    assert np.array_equal(s.D, Dn)
    d = s.r - rn
    d -= np.round(d / L) * L
    assert np.abs(d).max() <= 1e-12
    assert de == pytest.approx(den, rel=1e-9, abs=1e-9)
