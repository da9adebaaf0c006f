"""Engine (CUDA, through the C ABI) vs the FP64 oracle on identical draws.

Tolerances: the engine computes states, momenta and gradients in float32
with float64 log-densities/energies; the oracle is float64 throughout.
States/momenta after a transition must agree to 1e-5 relative (+1e-5
absolute); log-accept ratios to 2e-4 absolute; accept decisions and
leapfrog counts exactly, except on ties closer than those tolerances.
"""
import numpy as np
import pytest

from oracle import mcmc as omcmc
from oracle import philox, targets as otargets
from tests import _problems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def pg():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  return pg


def _logreg(pg, n, d, seed=0, scale=1.0):
  X, y, _ = _problems.logreg_data(n, d, seed, scale)
  return pg.LogisticRegression(X, y), otargets.LogisticRegression(X, y), X, y


@pytest.mark.parametrize('n,d,c', [(1000, 25, 64), (1003, 7, 70), (257, 100, 3), (64, 1, 1),
                                   (5000, 130, 129)])
def test_logreg_log_prob_and_grad(pg, n, d, c):
  t, o, _, _ = _logreg(pg, n, d, seed=n + d)
  q = np.random.default_rng(c).normal(size=(c, d)).astype(np.float32) * 0.3
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp_o, g_o = o(q)
  np.testing.assert_allclose(lp.cpu().numpy(), lp_o, rtol=2e-6, atol=1e-4)
  scale = np.abs(g_o).max()
  np.testing.assert_allclose(g.cpu().numpy(), g_o, rtol=1e-4, atol=2e-5 * scale)


def test_logreg_callable_matches_log_prob(pg):
  t, o, _, _ = _logreg(pg, 300, 5)
  q = np.zeros((4, 5), np.float32)
  np.testing.assert_allclose(t(torch.from_numpy(q).cuda()).cpu().numpy(), o(q)[0], rtol=1e-6)


def test_hmc_one_step_matches_oracle(pg):
  t, o, _, _ = _logreg(pg, 1000, 25, seed=0)
  C, D = 64, 25
  q0 = _problems.init_state(C, D)
  k = pg.mcmc.HamiltonianMonteCarlo(t, step_size=0.03, num_leapfrog_steps=10)
  kr = k.bootstrap_results(torch.from_numpy(q0).cuda())
  state = torch.from_numpy(q0).cuda()
  for step in range(3):
    seed = (1234, step)
    q_in = state.cpu().numpy()
    l_in = kr.accepted_results.target_log_prob.cpu().numpy()
    g_in = kr.accepted_results.grads_target_log_prob.cpu().numpy()
    state, kr = k.one_step(state, kr, seed=seed)
    r = omcmc.hmc_one_step(o, q_in, l_in, g_in, 0.03, 10, philox.PhiloxDraws(seed))
    p0 = kr.proposed_results.initial_momentum.cpu().numpy()
    np.testing.assert_allclose(p0, r.initial_momentum, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(kr.proposed_state.cpu().numpy(), r.proposed_state,
                               rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(kr.proposed_results.final_momentum.cpu().numpy(),
                               r.final_momentum, rtol=1e-5, atol=1e-5)
    lar = kr.log_accept_ratio.cpu().numpy()
    np.testing.assert_allclose(lar, r.log_accept_ratio, atol=2e-4)
    acc = kr.is_accepted.cpu().numpy()
    log_u = np.log(philox.uniform(seed, 'mh_uniform', C).astype(np.float64))
    tie = np.abs(log_u - r.log_accept_ratio) < 2e-4
    assert np.all((acc == r.is_accepted) | tie)
    keep = ~tie
    np.testing.assert_allclose(state.cpu().numpy()[keep], r.next_state[keep], rtol=1e-5,
                               atol=1e-5)


@pytest.mark.parametrize('depth,step', [(6, 0.05), (10, 0.02), (3, 0.2)])
def test_nuts_one_step_matches_oracle(pg, depth, step):
  t, o, _, _ = _logreg(pg, 1000, 25, seed=5)
  C, D = 48, 25
  q = torch.from_numpy(_problems.init_state(C, D, seed=3)).cuda()
  k = pg.mcmc.NoUTurnSampler(t, step_size=step, max_tree_depth=depth)
  kr = k.bootstrap_results(q)
  mism = 0
  for s in range(3):
    seed = (99, s)
    q_in = q.cpu().numpy()
    l_in = kr.target_log_prob.cpu().numpy()
    g_in = kr.grads_target_log_prob.cpu().numpy()
    q, kr = k.one_step(q, kr, seed=seed)
    r = omcmc.nuts_one_step(o, q_in, l_in, g_in, np.float32(step), philox.PhiloxDraws(seed),
                            depth)
    lf = kr.leapfrogs_taken.cpu().numpy()
    same = lf == r.leapfrogs_taken
    same &= kr.is_accepted.cpu().numpy() == r.is_accepted
    mism += int((~same).sum())
    np.testing.assert_allclose(q.cpu().numpy()[same], r.next_state[same], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(kr.log_accept_ratio.cpu().numpy()[same],
                               r.log_accept_ratio[same], atol=2e-4)
    np.testing.assert_allclose(kr.energy.cpu().numpy()[same], r.energy[same], rtol=1e-7,
                               atol=2e-4)
    np.testing.assert_array_equal(kr.has_divergence.cpu().numpy()[same], r.has_divergence[same])
    np.testing.assert_array_equal(kr.reach_max_depth.cpu().numpy()[same],
                                  r.reach_max_depth[same])
    # Continue both from the engine's state so later steps stay comparable.
  # Ties in U-turn dot products or uniforms may flip a rare chain.
  assert mism <= 2, mism


def test_nuts_per_chain_step_size(pg):
  t, o, _, _ = _logreg(pg, 500, 10, seed=8)
  C, D = 16, 10
  q = torch.from_numpy(_problems.init_state(C, D, seed=8)).cuda()
  eps = np.linspace(0.02, 0.2, C).astype(np.float32)
  k = pg.mcmc.NoUTurnSampler(t, step_size=torch.from_numpy(eps).cuda(), max_tree_depth=7)
  kr = k.bootstrap_results(q)
  q1, kr1 = k.one_step(q, kr, seed=(5, 5))
  r = omcmc.nuts_one_step(o, q.cpu().numpy(), kr.target_log_prob.cpu().numpy(),
                          kr.grads_target_log_prob.cpu().numpy(), eps, philox.PhiloxDraws((5, 5)), 7)
  same = kr1.leapfrogs_taken.cpu().numpy() == r.leapfrogs_taken
  assert same.sum() >= C - 1
  np.testing.assert_allclose(q1.cpu().numpy()[same], r.next_state[same], rtol=1e-5, atol=1e-5)


def test_nuts_reproducible(pg):
  t, _, _, _ = _logreg(pg, 800, 12, seed=2)
  q = torch.from_numpy(_problems.init_state(32, 12)).cuda()
  k = pg.mcmc.NoUTurnSampler(t, step_size=0.05, max_tree_depth=8)
  kr = k.bootstrap_results(q)
  a, ka = k.one_step(q, kr, seed=(1, 2))
  b, kb = k.one_step(q, kr, seed=(1, 2))
  assert torch.equal(a, b)
  assert torch.equal(ka.leapfrogs_taken, kb.leapfrogs_taken)


def test_dual_averaging_golden_constants_on_device(pg):
  # dual_averaging_step_size_adaptation_test.py:47-57 through the C ABI.
  from probability_gb300 import _native
  for err, expected in [(-0.05, 9.131008), (-0.02, 9.642897), (-0.01, 9.819825), (0.0, 10.0),
                        (0.01, 10.183481)]:
    lar = torch.full((4,), np.log(0.75 + err), dtype=torch.float64, device='cuda')
    state = torch.tensor([[0.0, 0.0, np.log(10.0), 0.0]], dtype=torch.float64, device='cuda')
    eps = torch.ones(1, dtype=torch.float32, device='cuda')
    ctx = _native.Context.current()
    _native.check(_native.lib().gbm_dual_averaging_update(
        ctx.handle, 4, _native.ptr(lar), 0, 10, 0.75, None, 0.05, 10.0, 0.75,
        _native.ptr(state), _native.ptr(eps)))
    np.testing.assert_allclose(eps.item(), expected, rtol=1e-6)


def test_sample_chain_nuts_dual_averaging_matches_oracle_steps(pg):
  """sample_chain(DA(NUTS)) step schedule and adapted step sizes against the
  oracle, transition by transition (the oracle re-started from the engine's
  state each step)."""
  t, o, _, _ = _logreg(pg, 600, 8, seed=11)
  C, D = 32, 8
  q0 = _problems.init_state(C, D, seed=11)
  nuts = pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=8)
  k = pg.mcmc.DualAveragingStepSizeAdaptation(nuts, num_adaptation_steps=6,
                                              target_accept_prob=0.8)
  res = pg.mcmc.sample_chain(num_results=9, current_state=torch.from_numpy(q0).cuda(),
                             kernel=k, num_burnin_steps=0, seed=(7, 7),
                             trace_fn=lambda s, kr: (kr.new_step_size,
                                                     kr.inner_results.log_accept_ratio,
                                                     kr.inner_results.seed),
                             return_final_kernel_results=True)
  assert res.all_states.shape == (9, C, D)
  assert res.final_kernel_results.step == 9
  steps = res.trace[0].cpu().numpy()
  lars = res.trace[1].cpu().numpy()
  seeds = res.trace[2].cpu().numpy()
  # The dual-averaging recursion, fed the engine's accept ratios.
  da = omcmc.DualAveraging(0.1, 6, 0.8)
  for i in range(9):
    da.update(lars[i])
    np.testing.assert_allclose(steps[i], da.new_step_size, rtol=1e-6)
  # Each recorded transition replays in the oracle from the previous state.
  states = np.concatenate([q0[None], res.all_states.cpu().numpy()])
  eps_used = np.concatenate([[0.1], steps[:-1]]).astype(np.float32)
  agree = 0
  for i in range(9):
    lp, g = o(states[i])
    r = omcmc.nuts_one_step(o, states[i], lp, g, eps_used[i],
                            philox.PhiloxDraws(tuple(seeds[i])), 8)
    ok = np.all(np.abs(r.next_state - states[i + 1]) <= 1e-5 + 1e-5 * np.abs(r.next_state), 1)
    agree += ok.sum()
  assert agree >= 9 * C - 3


def test_nan_initial_state_is_rejected_not_raised(pg):
  t, _, _, _ = _logreg(pg, 200, 4)
  q = torch.full((8, 4), float('nan'), device='cuda')
  k = pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=4)
  kr = k.bootstrap_results(q)
  q1, kr1 = k.one_step(q, kr, seed=(3, 3))
  assert not kr1.is_accepted.any()
  assert kr1.has_divergence.all()
