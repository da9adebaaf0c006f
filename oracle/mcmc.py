"""NumPy restatement of the reference's gradient-MCMC transition kernels.

Single state part, chain-major state ``[C, D]``, float64 by default (pass
``dtype=np.float32`` to mimic the reference's float32 arithmetic).  The
target is any callable ``f(state [C, D]) -> (logp [C], grad [C, D])`` from
``oracle.targets``.  Draws come from ``oracle.philox.PhiloxDraws``.

Chains are advanced in lock-step with per-chain masks, exactly as the
reference's batched ``tf.while_loop`` formulation does, so every mask rule of
the reference is exercised here.  Citations are relative to
``tensorflow_probability/python/``.
"""
import collections
import numpy as np

from oracle import philox

# --------------------------------------------------------------------------
# math helpers
# --------------------------------------------------------------------------


def log_add_exp(x, y):
  """math/generic.py:585-612: larger + softplus((x - larger) + (y - larger)).

  Like the reference, log_add_exp(-inf, -inf) is NaN.
  """
  with np.errstate(invalid='ignore'):
    larger = np.maximum(x, y)
    return larger + np.logaddexp(0.0, (x - larger) + (y - larger))


def reduce_logmeanexp(x, axis=None):
  """math/generic.py:221-275: log(mean(exp(x))) along ``axis``."""
  x = np.asarray(x, np.float64)
  m = np.max(x, axis=axis, keepdims=True)
  m = np.where(np.isfinite(m), m, 0.0)
  n = x.size if axis is None else np.prod([x.shape[a] for a in np.atleast_1d(axis)])
  out = np.log(np.sum(np.exp(x - m), axis=axis, keepdims=True)) + m - np.log(n)
  return np.squeeze(out, axis=axis) if axis is not None else out.reshape(())


def safe_sum(xs, alt_value=-np.inf):
  """mcmc/internal/util.py:205-235: elementwise sum, non-finite -> alt."""
  s = xs[0]
  for x in xs[1:]:
    s = s + x
  return np.where(np.isfinite(s), s, alt_value)


# --------------------------------------------------------------------------
# leapfrog (mcmc/internal/leapfrog_integrator.py:222-362)
# --------------------------------------------------------------------------


def leapfrog(target, p, q, logp, grad, eps, num_steps, dtype=np.float64, inv_mass=None):
  """SimpleLeapfrogIntegrator.__call__: half kick, num_steps x (drift, grad,
  kick), final -half kick correction (leapfrog_integrator.py:280-316,
  319-362).  ``eps`` broadcasts against ``[C, D]`` (per-chain step = [C, 1]).
  With ``inv_mass`` (diagonal M^-1), the drift moves by the velocity
  M^-1 p (leapfrog_integrator.py:267-275, 330-335).
  """
  eps = np.asarray(eps, dtype)
  half = np.asarray(0.5, dtype) * eps
  im = 1.0 if inv_mass is None else np.asarray(inv_mass, dtype)
  p_half = (p + half * grad).astype(dtype)
  for _ in range(num_steps):
    q = (q + eps * (p_half * im)).astype(dtype)
    logp, grad = target(q)
    logp = logp.astype(dtype)
    grad = grad.astype(dtype)
    p_half = (p_half + eps * grad).astype(dtype)
  p_new = (p_half - half * grad).astype(dtype)
  return p_new, q, logp, grad


# --------------------------------------------------------------------------
# HMC = MetropolisHastings(UncalibratedHamiltonianMonteCarlo)
# --------------------------------------------------------------------------

HMCStep = collections.namedtuple('HMCStep', [
    'next_state', 'target_log_prob', 'grads_target_log_prob',
    'proposed_state', 'proposed_target_log_prob', 'proposed_grads',
    'initial_momentum', 'final_momentum', 'log_acceptance_correction',
    'log_accept_ratio', 'is_accepted'])


def hmc_one_step(target, state, logp, grad, step_size, num_leapfrog_steps,
                 draws, dtype=np.float64):
  """hmc.py:661-729 (UncalibratedHMC) + metropolis_hastings.py:160-254."""
  C, D = state.shape
  state = state.astype(dtype)
  p0 = draws.momentum((C, D)).astype(dtype)                   # hmc.py:684-695
  eps = _chain_eps(step_size, C, dtype)
  p1, q1, l1, g1 = leapfrog(target, p0, state, logp.astype(dtype),
                            grad.astype(dtype), eps, num_leapfrog_steps, dtype)
  k0 = np.sum(p0 * p0, -1)
  k1 = np.sum(p1 * p1, -1)
  corr = np.asarray(0.5, dtype) * safe_sum([k0, -k1])          # hmc.py:861-875
  lar = safe_sum([l1, -logp.astype(dtype), corr])   # metropolis_hastings.py:204
  with np.errstate(divide='ignore'):
    log_u = np.log(draws.mh_uniform(C).astype(np.float64))
  acc = log_u < lar                                  # metropolis_hastings.py:221
  nxt = np.where(acc[:, None], q1, state)
  return HMCStep(nxt, np.where(acc, l1, logp), np.where(acc[:, None], g1, grad),
                 q1, l1, g1, p0, p1, corr, lar, acc)


def _chain_eps(step_size, C, dtype):
  s = np.asarray(step_size, dtype)
  if s.ndim == 0:
    return s
  return s.reshape(C, 1)


# --------------------------------------------------------------------------
# NUTS (nuts.py)
# --------------------------------------------------------------------------


def tree_uturn_instruction(max_depth):
  """nuts.py:1013-1028: (first leaf, last leaf) of every internal node of the
  depth-``max_depth`` tree whose leaves are numbered 0..2^depth-1, sorted."""
  pairs = []
  for h in range(1, max_depth + 1):
    size = 1 << h
    for a in range(0, 1 << max_depth, size):
      pairs.append((a, a + size - 1))
  return np.array(sorted(set(pairs)), dtype=np.int32).reshape(-1, 2)


def write_read_instruction(max_depth):
  """nuts.py:1031-1071: slot to write at each leaf, slot range to read.

  A leaf that starts a subtree of >= 2 leaves must keep its
  (momentum, momentum-cumsum) until the last leaf of the largest subtree it
  starts; its slot is the number of such saved leaves alive at that point
  minus one.  Leaves that start no subtree write a dummy slot (the maximum
  count), which is never read.  A leaf that ends subtrees checks every saved
  leaf starting one of them: a contiguous slot range [r0, r1).
  """
  instr = tree_uturn_instruction(max_depth)
  n = 1 << max_depth
  last_end = np.full(n, -1)
  ends_at = collections.defaultdict(list)
  for a, b in instr:
    last_end[a] = max(last_end[a], b)
    ends_at[b].append(a)
  alive_count = np.zeros(n, np.int64)
  for j in range(n):
    alive_count[j] = sum(1 for i in range(j + 1) if last_end[i] >= j)
  write = alive_count - 1
  dummy = alive_count.max()
  write[last_end < 0] = dummy
  read = np.zeros((n, 2), np.int64)
  for j in range(n):
    if ends_at[j]:
      alive = [i for i in range(j + 1) if last_end[i] >= j]
      r0 = alive.index(min(ends_at[j]))
      read[j] = (r0, r0 + len(ends_at[j]))
  return write, read


NUTSStep = collections.namedtuple('NUTSStep', [
    'next_state', 'target_log_prob', 'grads_target_log_prob',
    'log_accept_ratio', 'leapfrogs_taken', 'is_accepted', 'reach_max_depth',
    'has_divergence', 'energy', 'tree_depth'])


def _has_not_u_turn(diff, p_left, p_right):
  """nuts.py:987-1010 (generalised criterion, identity mass)."""
  return (np.sum(diff * p_left, -1) >= 0) & (np.sum(diff * p_right, -1) >= 0)


def nuts_one_step(target, state, logp, grad, step_size, draws, max_tree_depth=10,
                  max_energy_diff=1000.0, unrolled_leapfrog_steps=1,
                  dtype=np.float64, inv_mass=None):
  """NoUTurnSampler.one_step (nuts.py:321-445) with _loop_tree_doubling
  (:541-711), _build_sub_tree/_loop_build_sub_tree (:713-946) and
  has_not_u_turn_at_all_index (:949-984).  Multinomial sampling, generalised
  U-turn (the reference's static configuration, nuts.py:53-67).

  ``inv_mass`` (diagonal M^-1, [D] or [C, D]) gives PreconditionedNoUTurnSampler
  (experimental/mcmc/preconditioned_nuts.py:169) with the momentum
  distribution of preconditioning_utils.py:40-97 (precision = inv_mass):
  p = z / sqrt(inv_mass), kinetic energy 1/2 sum inv_mass p^2, drift by the
  velocity inv_mass p, U-turn dot products against velocities (:964-1030).
  The energy excludes the momentum distribution's normalizer."""
  C, D = state.shape
  write, read = write_read_instruction(max_tree_depth)
  n_slots = int(write.max()) + 1
  state = state.astype(dtype)
  logp = logp.astype(dtype)
  grad = grad.astype(dtype)
  s = np.asarray(step_size, dtype)
  eps_abs = np.full((C, 1), s, dtype) if s.ndim == 0 else s.reshape(C, 1)

  im = np.ones(D, dtype) if inv_mass is None else np.asarray(inv_mass, dtype)
  p0 = draws.momentum((C, D)).astype(dtype)                        # :512-529
  if inv_mass is not None:
    p0 = (p0 / np.sqrt(im)).astype(dtype)
  e0 = logp - 0.5 * np.sum(im * p0 * p0, -1)                        # :1085-1102
  # trajectory ends [left, right] (:352-361)
  ends = dict(p=np.stack([p0, p0]), q=np.stack([state, state]),
              l=np.stack([logp, logp]), g=np.stack([grad, grad]))
  cand = dict(q=state.copy(), l=logp.copy(), g=grad.copy(), e=e0.copy(),
              w=np.zeros(C))
  is_accepted = np.zeros(C, bool)
  momentum_sum = p0.copy()
  energy_diff_sum = np.zeros(C)
  leapfrog_count = np.zeros(C, np.int64)
  continue_tree = np.ones(C, bool)
  not_divergence = np.ones(C, bool)
  tree_depth = np.zeros(C, np.int64)
  slot_p = np.zeros((n_slots, C, D), dtype)
  slot_cs = np.zeros((n_slots, C, D), dtype)
  ar = np.arange(C)

  for depth in range(max_tree_depth):                               # :404-422
    if not continue_tree.any():
      break
    tree_depth += continue_tree
    fwd = draws.direction(C, depth).astype(bool)                    # :551-558
    side = fwd.astype(np.int64)                  # 1: extend right, 0: left
    eps = np.where(fwd[:, None], eps_abs, -eps_abs)
    cur = {k: v[side, ar] for k, v in ends.items()}                 # :560-562
    sub_w = np.full(C, -np.inf)                                     # :727-731
    sub = dict(q=cur['q'].copy(), l=cur['l'].copy(), g=cur['g'].copy(),
               e=cur['l'].copy())
    cumsum = np.zeros((C, D), dtype)
    sub_eds = np.zeros(C)
    sub_lf = np.zeros(C, np.int64)
    sub_cont = continue_tree.copy()
    sub_nd = not_divergence.copy()

    for leaf in range(1 << depth):                                  # :761-791
      if not sub_cont.any():
        break
      p1, q1, l1, g1 = leapfrog(target, cur['p'], cur['q'], cur['l'], cur['g'],
                                eps, unrolled_leapfrog_steps, dtype,
                                None if inv_mass is None else im)
      cumsum_prev = cumsum
      cumsum = cumsum + p1                                          # :827-828
      sub_lf = np.where(sub_cont, sub_lf + 1, sub_lf)               # :829-830
      no_uturn = np.ones(C, bool)                                   # :846-855
      v1 = p1 * im                                                  # velocity
      for i in range(int(read[leaf, 0]), int(read[leaf, 1])):
        diff = cumsum - slot_cs[i]
        no_uturn &= _has_not_u_turn(diff, slot_p[i], v1)
      w = int(write[leaf])                                          # :857-869
      slot_p[w] = v1
      slot_cs[w] = cumsum_prev
      energy = l1.astype(np.float64) - 0.5 * np.sum(
          im * p1.astype(np.float64) ** 2, -1)                      # :871-876
      energy = np.where(np.isnan(energy), -np.inf, energy)
      with np.errstate(invalid='ignore'):
        energy_diff = energy - e0
        not_div = -energy_diff < max_energy_diff                    # :880
        weight_sum = log_add_exp(sub_w, energy_diff)                # :881-883
        thresh = energy_diff - weight_sum
      u = np.log1p(-draws.leaf_uniform(C, depth, leaf).astype(np.float64))
      with np.errstate(invalid='ignore'):
        acc = u <= thresh                                           # :901
      sub['q'] = np.where(acc[:, None], q1, sub['q'])
      sub['l'] = np.where(acc, l1, sub['l'])
      sub['g'] = np.where(acc[:, None], g1, sub['g'])
      sub['e'] = np.where(acc, energy, sub['e'])
      sub_w = weight_sum
      cont = not_div & sub_cont                                     # :921-933
      nd_keep = np.where(sub_cont, not_div, True)
      with np.errstate(invalid='ignore'):
        sub_eds = np.where(cont, sub_eds + np.exp(np.minimum(energy_diff, 0.0)),
                           sub_eds)
      sub_nd = sub_nd & nd_keep
      sub_cont = no_uturn & cont
      cur = dict(p=p1, q=q1, l=l1, g=g1)

    # tree-level biased progressive sampling (:597-642)
    energy_diff_sum = energy_diff_sum + sub_eds
    tree_w = np.where(sub_cont, sub_w, -np.inf)
    weight_sum = log_add_exp(tree_w, cand['w'])
    with np.errstate(invalid='ignore'):
      thresh = tree_w - cand['w']
    thresh = np.where(np.isnan(thresh), 0.0, thresh)
    u = np.log1p(-draws.tree_uniform(C, depth).astype(np.float64))
    choose = (u <= thresh) & sub_cont
    for k in ('q', 'g'):
      cand[k] = np.where(choose[:, None], sub[k], cand[k])
    for k in ('l', 'e'):
      cand[k] = np.where(choose, sub[k], cand[k])
    cand['w'] = weight_sum
    # trajectory ends and trajectory-level U-turn (:653-709)
    for k in ends:
      ends[k][side, ar] = cur[k]
    momentum_sum = momentum_sum + cumsum
    no_uturn_traj = _has_not_u_turn(momentum_sum, ends['p'][0] * im, ends['p'][1] * im)
    is_accepted = choose | is_accepted
    continue_tree = sub_cont & no_uturn_traj
    not_divergence = sub_nd
    leapfrog_count = leapfrog_count + sub_lf

  with np.errstate(divide='ignore', invalid='ignore'):
    lar = np.log(energy_diff_sum / leapfrog_count)                  # :429-432
  return NUTSStep(cand['q'], cand['l'], cand['g'], lar,
                  leapfrog_count * unrolled_leapfrog_steps, is_accepted,
                  continue_tree, ~not_divergence, cand['e'], tree_depth)


# --------------------------------------------------------------------------
# Dual averaging (dual_averaging_step_size_adaptation.py:353-609)
# --------------------------------------------------------------------------

class DualAveraging:
  """Step-size state of DualAveragingStepSizeAdaptation for one step-size
  part.  ``step_size`` is a scalar (shared; the chain axis is reduced with
  reduce_logmeanexp, :411-418) or ``[C]`` (per chain; no reduction)."""

  def __init__(self, step_size, num_adaptation_steps, target_accept_prob=0.75,
               exploration_shrinkage=0.05, shrinkage_target=None,
               step_count_smoothing=10, decay_rate=0.75):
    self.step_size = np.asarray(step_size, np.float64)
    self.num_adaptation_steps = int(num_adaptation_steps)
    self.target_accept_prob = np.asarray(target_accept_prob, np.float64)
    self.exploration_shrinkage = float(exploration_shrinkage)
    self.step_count_smoothing = float(step_count_smoothing)
    self.decay_rate = float(decay_rate)
    if shrinkage_target is None:                                    # :588-590
      self.log_shrinkage_target = np.log(10.0) + np.log(self.step_size)
    else:
      self.log_shrinkage_target = np.log(np.asarray(shrinkage_target, np.float64))
    self.error_sum = np.zeros_like(self.step_size)
    self.log_averaging_step = np.zeros_like(self.step_size)
    self.step = 0
    self.new_step_size = self.step_size.copy()

  @staticmethod
  def log_accept_prob(log_accept_ratio):
    """simple_step_size_adaptation.py:42-48: min(lar, 0), non-finite->-inf."""
    lar = np.asarray(log_accept_ratio, np.float64)
    return np.minimum(np.where(np.isfinite(lar), lar, -np.inf), 0.0)

  def update(self, log_accept_ratio):
    """_one_step_part (:353-475) after the inner kernel ran with
    ``self.new_step_size`` (the setter, :482-485)."""
    step_size = self.new_step_size
    lap = self.log_accept_prob(log_accept_ratio)
    red = reduce_logmeanexp(lap) if step_size.ndim == 0 else lap
    new_error_sum = self.error_sum + self.target_accept_prob - np.exp(red)
    step = float(self.step) + 1.0
    soft_t = self.step_count_smoothing + step
    new_log_step = self.log_shrinkage_target - (
        new_error_sum * np.sqrt(step)) / (soft_t * self.exploration_shrinkage)
    eta = step ** (-self.decay_rate)
    new_log_avg = eta * new_log_step + (1.0 - eta) * self.log_averaging_step
    istep = self.step + 1
    if istep < self.num_adaptation_steps:
      new_step = np.exp(new_log_step)
    elif istep > self.num_adaptation_steps:
      new_step = step_size
    else:
      new_step = np.exp(new_log_avg)
    if istep > self.num_adaptation_steps:
      new_log_avg = self.log_averaging_step
    self.error_sum = new_error_sum
    self.log_averaging_step = new_log_avg
    self.new_step_size = np.asarray(new_step, np.float64)
    self.step = istep
    return self.new_step_size


# --------------------------------------------------------------------------
# sample_chain (sample.py:311-383)
# --------------------------------------------------------------------------

def num_transitions(num_results, num_burnin_steps=0, num_steps_between_results=0):
  """sample.py:359-367: result 0 after 1 + burnin steps, then 1 + thin."""
  return num_burnin_steps + 1 + (num_results - 1) * (1 + num_steps_between_results)


def sample_chain_nuts(target, init_state, seed, num_results, num_burnin_steps,
                      step_size, num_adaptation_steps=None,
                      target_accept_prob=0.75, max_tree_depth=10,
                      num_steps_between_results=0, dtype=np.float64):
  """sample_chain(DualAveragingStepSizeAdaptation(NoUTurnSampler)) with the
  engine's per-step key schedule (philox.step_key(seed, t))."""
  state = np.asarray(init_state, dtype)
  logp, grad = target(state)
  da = None
  if num_adaptation_steps is not None:
    da = DualAveraging(step_size, num_adaptation_steps, target_accept_prob)
  eps = np.asarray(step_size, np.float64)
  out_states, out_lar, out_lf = [], [], []
  total = num_transitions(num_results, num_burnin_steps, num_steps_between_results)
  result_at = set(num_burnin_steps + i * (1 + num_steps_between_results)
                  for i in range(num_results))
  for t in range(total):
    draws = philox.PhiloxDraws(philox.step_key(seed, t))
    eps_t = da.new_step_size if da is not None else eps
    r = nuts_one_step(target, state, logp, grad, eps_t.astype(np.float32),
                      draws, max_tree_depth, dtype=dtype)
    state, logp, grad = r.next_state, r.target_log_prob, r.grads_target_log_prob
    if da is not None:
      da.update(r.log_accept_ratio)
    if t in result_at:
      out_states.append(state.copy())
      out_lar.append(r.log_accept_ratio)
      out_lf.append(r.leapfrogs_taken)
  return np.stack(out_states), np.stack(out_lar), np.stack(out_lf)
