"""GPU MCMC relocation + growth (Model::mcmcAfterTrain, core/src/model.cpp:
497-660) against the oracle.

The draws come from a different random stream than the reference's
std::mt19937 + discrete_distribution, so parity is checked in two parts:
  * given the (dst, src) pairs the device chose, every parameter and Adam
    moment equals the oracle's relocate/addNewGaussians applied to the same
    pairs (model.cpp:380-416, 465-491);
  * the choice itself has the reference's distribution: dead slots are
    exactly the oracle's dead mask, sources are alive, and source
    frequencies follow sigmoid(opacity) (chi-square)."""
import numpy as np
import pytest

from msplat_gb300 import engine as E
from msplat_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _scene(n, seed, dead_frac=0.2, nan_rows=7, far_rows=11):
    rng = np.random.default_rng(seed)
    g = S.gaussians(n, seed=seed, sh_rest_bases=15)
    g.opacities[:] = rng.normal(0.0, 1.5, n).astype(np.float32).reshape(g.opacities.shape)
    op = g.opacities.reshape(-1)
    perm = rng.permutation(n)                              # disjoint dead / non-finite / far rows
    k = int(dead_frac * n)
    dead, bad, far = perm[:k], perm[k:k + nan_rows], perm[k + nan_rows:k + nan_rows + far_rows]
    op[dead] = -8.0                                       # sigmoid < 0.005
    g.features_rest.reshape(n, -1)[bad, 5] = np.nan        # non-finite
    g.means[far] = np.array([9.0, 0.0, 0.0], np.float32)   # outside the cull radius
    return g


def _moments(dg, seed):
    import torch
    gen = torch.Generator(device="cuda").manual_seed(seed)
    for d in (dg.exp_avg, dg.exp_avg_sq):
        for k, t in d.items():
            t.copy_(torch.rand(t.shape, generator=gen, device="cuda"))


def _host_state(dg):
    p, (m, v) = dg.to_numpy(rows=dg.cap)
    g = S.GaussianSet(*(p[k].copy() for k in E.GROUPS))
    return g, ([m[k].copy() for k in E.GROUPS], [v[k].copy() for k in E.GROUPS])


def _run(n, cap, seed, cull=3.0, **kw):
    init = _scene(n, seed, **kw)
    dg = E.DeviceGaussians(init, cap=cap)
    _moments(dg, seed)
    before, mom_before = _host_state(dg)
    eng = E.Engine(0, cap)
    stats, rc = eng.mcmc(dg, cull, 10)
    moves = eng.read("mcmc_moves", np.int32, 2 * (stats.num_relocated + stats.num_grown)).reshape(-1, 2)
    after, mom_after = _host_state(dg)
    eng.close()
    return init, before, mom_before, stats, rc, moves, after, mom_after


def test_mcmc_matches_oracle_given_moves():
    n, cap = 20000, 40000
    init, before, mom, stats, rc, moves, after, mom_after = _run(n, cap, seed=3)
    dead_mask, cnt = O.mcmc_dead_mask(init, 3.0)
    assert stats.num_dead == cnt
    assert stats.num_nonfinite == 7
    assert stats.num_culled == 11
    assert rc == 12                                           # one seed for relocation, one for growth
    assert stats.num_relocated == cnt
    assert stats.num_grown == int(np.float32(1.05) * np.float32(n)) - n   # (int)(1.05f * N)
    assert stats.num_active == n + stats.num_grown
    reloc, grow = moves[:stats.num_relocated], moves[stats.num_relocated:]
    # relocation targets are exactly the dead slots, sources are alive
    assert np.array_equal(np.sort(reloc[:, 0]), np.flatnonzero(dead_mask))
    assert not dead_mask[reloc[:, 1]].any()
    # growth fills n, n+1, ... from the (post-relocation) first n rows
    assert np.array_equal(grow[:, 0], np.arange(n, n + stats.num_grown))
    assert (grow[:, 1] >= 0).all() and (grow[:, 1] < n).all()

    ref, ref_mom = before, mom
    O.mcmc_apply(ref, ref_mom, reloc[:, 0], reloc[:, 1])
    O.mcmc_apply(ref, ref_mom, grow[:, 0], grow[:, 1])
    rows = stats.num_active
    for k, a, b in zip(E.GROUPS, after.arrays(), ref.arrays()):
        a, b = a[:rows], b[:rows]
        if k in ("opacities", "scales"):
            # Eq. 9 through device expf/logf/powf vs the host's: a few ulp
            np.testing.assert_allclose(a, b, rtol=2e-6, atol=2e-6, err_msg=k)
        else:
            assert np.array_equal(a, b, equal_nan=True), k
    for gi, k in enumerate(E.GROUPS):
        assert np.array_equal(mom_after[0][gi][:rows], ref_mom[0][gi][:rows]), k
        assert np.array_equal(mom_after[1][gi][:rows], ref_mom[1][gi][:rows]), k
    # rows past the active count are untouched
    for a, b in zip(after.arrays(), before.arrays()):
        assert np.array_equal(a[rows:], b[rows:])
    # no non-finite or culled row survives relocation
    assert np.isfinite(after.features_rest[:rows]).all()
    assert (np.square(after.means[:rows]).sum(1) <= 9.0).all()


def test_mcmc_sampling_follows_opacity():
    """Half the slots dead; the living have sigmoid(opacity) in four levels.
    Relocation draws 8192 sources: their level histogram must match the
    weight shares (chi-square, 3 dof, far tail)."""
    n = 16384
    g = S.gaussians(n, seed=5, sh_rest_bases=0)
    levels = np.array([0.1, 0.3, 0.6, 0.9], np.float32)
    op = g.opacities.reshape(-1)
    lvl = np.arange(n) % 8                      # odd positions dead, even ones in 4 levels
    alive = lvl % 2 == 0
    op[~alive] = -9.0
    lv = (lvl // 2).astype(np.int64)
    op[alive] = np.log(levels[lv[alive]] / (1 - levels[lv[alive]]))
    g.means[:] = np.clip(g.means, -1, 1)
    dg = E.DeviceGaussians(g, cap=n)              # cap = n: no growth
    eng = E.Engine(0, n)
    stats, _ = eng.mcmc(dg, 0.0, 0)
    assert stats.num_dead == n // 2 and stats.num_grown == 0
    moves = eng.read("mcmc_moves", np.int32, 2 * stats.num_relocated).reshape(-1, 2)
    eng.close()
    src = moves[:, 1]
    assert alive[src].all()
    obs = np.bincount(lv[src], minlength=4).astype(np.float64)
    share = levels * (n // 8)
    exp = share / share.sum() * len(src)
    chi2 = float(((obs - exp) ** 2 / exp).sum())
    assert chi2 < 35.0, (obs, exp, chi2)       # p ~ 1e-7 for 3 dof


def test_mcmc_nothing_dead_grows_only():
    n = 4096
    g = S.gaussians(n, seed=9, sh_rest_bases=3)
    g.opacities[:] = 0.5
    g.means[:] = np.clip(g.means, -1, 1)
    dg = E.DeviceGaussians(g, cap=n + 100)
    eng = E.Engine(0, n + 100)
    stats, rc = eng.mcmc(dg, 3.0, 0)
    eng.close()
    assert stats.num_dead == 0 and stats.num_relocated == 0
    assert stats.num_grown == 100 and dg.n == n + 100     # capped at cap_max
    assert rc == 1


def _mix32(seed, idx):
    """The engine's counter hash (PCG output step on seed*747796405 + idx*2891336453), vectorised."""
    x = (np.uint64(seed) * np.uint64(747796405) + idx.astype(np.uint64) * np.uint64(2891336453)) & np.uint64(0xFFFFFFFF)
    x = (((x >> ((x >> np.uint64(28)) + np.uint64(4))) ^ x) * np.uint64(277803737)) & np.uint64(0xFFFFFFFF)
    return (x >> np.uint64(22)) ^ x


def _unit53(seed, j):
    hi = _mix32(seed, 2 * j)
    lo = _mix32(seed ^ 0x85EBCA6B, 2 * j + 1)
    bits = ((hi << np.uint64(32)) | lo) >> np.uint64(11)
    return bits.astype(np.float64) * (1.0 / 9007199254740992.0)


def test_mcmc_draws_exact_and_64_levels():
    """Every relocation draw equals the first index whose cumulative weight
    exceeds u * total, u the 53-bit counter-based uniform of that draw (an
    exact restatement on the device's own cumulative weights: no off-by-one
    at bucket edges); the weights are the living Gaussians' sigmoid(opacity)
    and the cumulative weights their running sum; and the sources of 16,384
    draws over 64 graded opacity levels pass a 63-dof chi-square test."""
    n = 32768
    g = S.gaussians(n, seed=6, sh_rest_bases=0)
    levels = np.linspace(0.02, 0.98, 64).astype(np.float32)
    op = g.opacities.reshape(-1)
    alive = np.arange(n) % 2 == 0
    lv = (np.arange(n) // 2) % 64
    op[~alive] = -9.0
    op[alive] = np.log(levels[lv[alive]] / (1 - levels[lv[alive]]))
    g.means[:] = np.clip(g.means, -1, 1)
    dg = E.DeviceGaussians(g, cap=n)
    eng = E.Engine(0, n)
    stats, rc = eng.mcmc(dg, 0.0, 0)
    assert stats.num_dead == n // 2 and stats.num_relocated == n // 2 and stats.num_grown == 0
    moves = eng.read("mcmc_moves", np.int32, 2 * stats.num_relocated).reshape(-1, 2)
    w = eng.read("mcmc_weights", np.float64, n)
    cumw = eng.read("mcmc_cumw", np.float64, n)
    eng.close()
    sig = (1.0 / (1.0 + np.exp(-op.astype(np.float64)))).astype(np.float32)
    ref_w = np.where(alive, sig, 0.0)
    np.testing.assert_allclose(w, ref_w, rtol=3e-7, atol=0)
    np.testing.assert_allclose(cumw, np.cumsum(w), rtol=1e-12, atol=0)
    seed = 0x9E3779B9 ^ 1                      # the first relocation round of a run
    j = np.arange(stats.num_relocated, dtype=np.uint64)
    target = _unit53(seed, j) * cumw[-1]
    expect = np.searchsorted(cumw, target, side="right")
    assert np.array_equal(moves[:, 1], expect)
    src = moves[:, 1]
    assert alive[src].all()
    obs = np.bincount(lv[src], minlength=64).astype(np.float64)
    exp = levels / levels.sum() * len(src)
    chi2 = float(((obs - exp) ** 2 / exp).sum())
    try:
        from scipy.stats import chi2 as C2
        bar = float(C2.isf(1e-6, 63))
    except ImportError:   # the 1e-6 tail of 63 dof
        bar = 131.4
    assert chi2 < bar, (chi2, bar)
