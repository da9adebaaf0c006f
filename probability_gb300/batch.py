"""Many independent posteriors of uneven dimension in one NUTS sampler.

``TargetBatch([(target, chains), ...])`` concatenates the chains of several
multivariate-normal and non-centred hierarchical-normal posteriors into one
ragged population (C-ABI ``gbm_target_batch``); ``BatchedNoUTurnSampler``
runs the reference's NoUTurnSampler transition (mcmc/nuts.py:321-445) on all
of them at once, with a step size per member.  States, gradients and momenta
are flat float32 vectors: member t's chains follow member t-1's and chain c's
vector occupies ``offsets[c] : offsets[c] + dims[c]``; ``pack`` and
``unpack`` convert from and to per-member ``[chains, dim]`` tensors.

Every sampler step launches the same kernels whatever the number of members:
the per-leaf gradient is two persistent launches over a device-built tile
list, and batches of leaves are replayed as CUDA graphs.  The chain-tile width of each size class of D is picked by
timing at construction (``schedule``).
"""
import ctypes

import numpy as np
import torch

from probability_gb300 import _native, _util, targets
from probability_gb300.mcmc.nuts import NUTSKernelResults

FAMILY_MVN, FAMILY_HIER = 1, 2
P = ctypes.c_void_p


class BatchMember(ctypes.Structure):
  _fields_ = [('family', ctypes.c_int32), ('dim', ctypes.c_int64), ('chains', ctypes.c_int64),
              ('loc', P), ('scale_tril_inv', P), ('log_normalizer', ctypes.c_double),
              ('group_y', P), ('group_sigma', P), ('mu_scale', ctypes.c_float),
              ('tau_scale', ctypes.c_float)]


_SIGS = {
    'gbm_target_batch': ([P, ctypes.POINTER(BatchMember), ctypes.c_int64, ctypes.POINTER(P)],
                         ctypes.c_int),
    'gbm_target_batch_layout': ([P, P, P, ctypes.POINTER(ctypes.c_int64),
                                 ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    'gbm_target_batch_schedule': ([P, ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
}


def _lib():
  L = _native.lib()
  if not getattr(L, '_batch_sigs', False):
    for name, (args, res) in _SIGS.items():
      fn = getattr(L, name)
      fn.argtypes = args
      fn.restype = res
    L._batch_sigs = True
  return L


class TargetBatch(targets.Target):
  """A ragged batch of posteriors: ``members`` is a list of ``(target,
  chains)`` with ``target`` a MultivariateNormalTriL or a
  NonCentredHierarchicalNormal."""

  def __init__(self, members, stream=None):
    dev = _util.device()
    # The batch's own stream (work of the batch is ordered on it).
    self.stream = torch.cuda.Stream(dev) if stream is None else stream
    self.stream.wait_stream(torch.cuda.current_stream(dev))
    arr = (BatchMember * len(members))()
    keep = []
    for i, (t, c) in enumerate(members):
      m = arr[i]
      m.chains = int(c)
      if isinstance(t, targets.MultivariateNormalTriL):
        m.family, m.dim = FAMILY_MVN, t.event_dim
        m.loc, m.scale_tril_inv = _native.ptr(t._loc_t), _native.ptr(t._linv_t)
        m.log_normalizer = t._log_norm
      elif isinstance(t, targets.NonCentredHierarchicalNormal):
        m.family, m.dim = FAMILY_HIER, t.groups
        m.group_y, m.group_sigma = _native.ptr(t._y_t), _native.ptr(t._s_t)
        m.mu_scale, m.tau_scale = t.mu_scale, t.tau_scale
      else:
        raise NotImplementedError('TargetBatch members are MultivariateNormalTriL or '
                                  'NonCentredHierarchicalNormal targets')
      keep.append(t)
    with torch.cuda.stream(self.stream):
      ctx = _native.Context.current()
      h = P()
      _native.check(_lib().gbm_target_batch(ctx.handle, arr, len(members), ctypes.byref(h)),
                    'gbm_target_batch')
    self._handle = h
    self._ctx = ctx
    self.members = keep
    self.member_chains = [int(c) for _, c in members]
    C, E = ctypes.c_int64(), ctypes.c_int64()
    _native.check(_lib().gbm_target_batch_layout(h, None, None, ctypes.byref(C), ctypes.byref(E)),
                  'gbm_target_batch_layout')
    self.chains, self.elements = int(C.value), int(E.value)
    off = np.empty(self.chains, np.int64)
    dims = np.empty(self.chains, np.int32)
    _native.check(_lib().gbm_target_batch_layout(
        h, off.ctypes.data_as(P), dims.ctypes.data_as(P), None, None), 'gbm_target_batch_layout')
    self.offsets, self.dims = off, dims
    self.member_dims = [t.event_dim for t in keep]
    self.chain_begin = np.concatenate([[0], np.cumsum(self.member_chains)]).astype(np.int64)
    self.elem_begin = off[self.chain_begin[:-1]]

  def schedule(self):
    """Chain tile chosen by the autotuner for MVN members with D <= 64, <= 256,
    <= 1024, > 1024 (0: no member in that class)."""
    ct = (ctypes.c_int32 * 4)()
    _native.check(_lib().gbm_target_batch_schedule(self._handle, ct), 'gbm_target_batch_schedule')
    return dict(zip(['d<=64', 'd<=256', 'd<=1024', 'd>1024'], list(ct)))

  def pack(self, per_member):
    """Per-member [chains_t, dim_t] tensors -> the flat ragged vector."""
    return torch.cat([_util.as_tensor(x, torch.float32).reshape(-1) for x in per_member])

  def unpack(self, flat):
    """The flat ragged vector -> per-member [chains_t, dim_t] views."""
    out = []
    for t in range(len(self.members)):
      e0 = int(self.elem_begin[t])
      n = self.member_chains[t] * self.member_dims[t]
      out.append(flat[e0:e0 + n].view(self.member_chains[t], self.member_dims[t]))
    return out

  def per_chain(self, per_member_values, dtype=torch.float32):
    """One value per member -> one per chain."""
    dev = _util.device()
    v = torch.as_tensor(per_member_values, dtype=dtype).to(dev)
    return torch.repeat_interleave(v, torch.as_tensor(self.member_chains, device=dev))

  def _enter(self):
    self.stream.wait_stream(torch.cuda.current_stream(self.stream.device))

  def _leave(self):
    torch.cuda.current_stream(self.stream.device).wait_stream(self.stream)

  def log_prob_and_grad(self, state):
    q = _util.as_tensor(state, torch.float32).reshape(-1)
    if q.numel() != self.elements:
      raise ValueError('state must hold %d elements (the ragged layout)' % self.elements)
    logp = torch.empty(self.chains, dtype=torch.float64, device=q.device)
    grad = torch.empty_like(q)
    self._enter()
    _native.check(_native.lib().gbm_target_log_prob_and_grad(
        self._handle, _native.ptr(q), self.chains, _native.ptr(logp), _native.ptr(grad)),
        'gbm_target_log_prob_and_grad')
    self._leave()
    return logp, grad


class BatchedNoUTurnSampler:
  """NoUTurnSampler (mcmc/nuts.py:165) over every chain of a TargetBatch;
  ``step_size`` is one value per member (or per chain)."""

  def __init__(self, batch, step_size, max_tree_depth=10, max_energy_diff=1000.,
               unrolled_leapfrog_steps=1, use_graphs=True):
    if not isinstance(batch, TargetBatch):
      raise TypeError('BatchedNoUTurnSampler samples a TargetBatch')
    self.batch = batch
    self.max_tree_depth = int(max_tree_depth)
    self.step_size = step_size
    h = P()
    _native.check(_native.lib().gbm_nuts_create(
        batch._handle, batch.chains, self.max_tree_depth, float(max_energy_diff),
        int(unrolled_leapfrog_steps), ctypes.byref(h)), 'gbm_nuts_create')
    self._handle = h
    _native.check(_native.lib().gbm_nuts_set_graphs(h, int(bool(use_graphs))),
                  'gbm_nuts_set_graphs')
    self.last_leaf_iterations = 0
    self.inverse_mass = None

  def set_inverse_mass(self, inverse_mass):
    """Diagonal inverse mass matrix (the preconditioning of
    PreconditionedNoUTurnSampler) for the following steps: a ragged float32
    vector with one entry per state element, or None for the identity."""
    if inverse_mass is None:
      self.inverse_mass = None
      ptr = None
    else:
      v = _util.as_tensor(inverse_mass, torch.float32).reshape(-1).contiguous()
      if v.numel() != self.batch.elements:
        raise ValueError('inverse_mass needs one entry per state element')
      self.inverse_mass = v              # kept alive while the engine reads it
      ptr = _native.ptr(v)
    _native.check(_native.lib().gbm_nuts_set_inverse_mass(self._handle, ptr, 1),
                  'gbm_nuts_set_inverse_mass')

  def __del__(self):
    if getattr(self, '_handle', None) is not None and _native._lib is not None:
      try:
        _native.lib().gbm_nuts_destroy(self._handle)
      except Exception:
        pass

  def _eps(self, step_size):
    s = torch.as_tensor(step_size, dtype=torch.float32).reshape(-1)
    if s.numel() == len(self.batch.members):
      return self.batch.per_chain(s)
    if s.numel() == self.batch.chains:
      return s.to(_util.device())
    raise ValueError('step_size needs one value per member or per chain')

  def bootstrap_results(self, init_state):
    q = _util.as_tensor(init_state, torch.float32).reshape(-1)
    logp, grad = self.batch.log_prob_and_grad(q)
    C = self.batch.chains
    z = lambda dt: torch.zeros(C, dtype=dt, device=q.device)
    return NUTSKernelResults(
        target_log_prob=logp, grads_target_log_prob=grad, step_size=self._eps(self.step_size),
        log_accept_ratio=z(torch.float64), leapfrogs_taken=z(torch.int32),
        is_accepted=z(torch.bool), reach_max_depth=z(torch.bool), has_divergence=z(torch.bool),
        energy=logp.clone(), seed=_util.seed_tensor((0, 0)))

  def one_step(self, current_state, previous_kernel_results, seed=None):
    seed = _util.sanitize_seed(seed)
    b = self.batch
    q = _util.as_tensor(current_state, torch.float32).reshape(-1)
    pkr = previous_kernel_results
    C, dev = b.chains, q.device
    eps = self._eps(pkr.step_size)
    nq, ng = torch.empty_like(q), torch.empty_like(q)
    f64 = lambda: torch.empty(C, dtype=torch.float64, device=dev)
    u8 = lambda: torch.empty(C, dtype=torch.uint8, device=dev)
    nl, lar, energy = f64(), f64(), f64()
    lf = torch.empty(C, dtype=torch.int32, device=dev)
    acc, rmd, div = u8(), u8(), u8()
    Pt = _native.ptr
    b._enter()
    _native.check(_native.lib().gbm_nuts_one_step(
        self._handle, C, Pt(q), Pt(pkr.target_log_prob), Pt(pkr.grads_target_log_prob), Pt(eps),
        1, _native.seed_words(seed), Pt(nq), Pt(nl), Pt(ng), Pt(lar), Pt(lf), Pt(acc), Pt(rmd),
        Pt(div), Pt(energy), None), 'gbm_nuts_one_step')
    b._leave()
    n = ctypes.c_int64()
    _native.lib().gbm_nuts_last_leaf_iterations(self._handle, ctypes.byref(n))
    self.last_leaf_iterations = int(n.value)
    return nq, NUTSKernelResults(
        target_log_prob=nl, grads_target_log_prob=ng, step_size=eps, log_accept_ratio=lar,
        leapfrogs_taken=lf, is_accepted=acc.bool(), reach_max_depth=rmd.bool(),
        has_divergence=div.bool(), energy=energy, seed=_util.seed_tensor(seed))

  def run_free(self, current_state, kernel_results, transitions_per_chain, seed,
                 first_step=0, max_leaf_iterations=1 << 40):
    """Free-running transitions of every member's chains (no lock-step
    across chains or members: a chain starts its next transition as soon as
    its own trajectory ends), per chain equal to one_step with keys
    step_key(seed, first_step + t).  Returns FreeRun(all_states [K, elements]
    (ragged, as the state), trace of [K, chains] tensors, transitions_done,
    leaf_iterations)."""
    from probability_gb300.mcmc.nuts import run_free
    b = self.batch
    q = _util.as_tensor(current_state, torch.float32).reshape(-1).contiguous()
    eps = self._eps(kernel_results.step_size).contiguous()
    b._enter()
    try:
      run = run_free(self._handle, q, kernel_results, eps, 1, _util.sanitize_seed(seed),
                     first_step, transitions_per_chain, max_leaf_iterations, (q.numel(),))
    finally:
      b._leave()
    self.last_leaf_iterations = run.leaf_iterations
    return run


class MemberMassMatrixAdaptation:
  """DiagonalMassMatrixAdaptation (experimental/mcmc/
  diagonal_mass_matrix_adaptation.py:73) for every member of a batch: the
  running variance of each member's state, per dimension, with every chain
  and step a sample, expanded to the ragged per-element inverse mass.  Two
  scatter-adds per update whatever the number of members."""

  def __init__(self, batch):
    dev = _util.device()
    self.batch = batch
    g, base = [], 0
    for c, d in zip(batch.member_chains, batch.member_dims):
      g.append(np.tile(np.arange(base, base + d), c))
      base += d
    self.groups = base
    self.index = torch.from_numpy(np.concatenate(g)).to(dev)
    self.reset()

  def reset(self):
    dev = self.index.device
    self.s1 = torch.zeros(self.groups, dtype=torch.float64, device=dev)
    self.s2 = torch.zeros(self.groups, dtype=torch.float64, device=dev)
    self.count = torch.zeros(self.groups, dtype=torch.float64, device=dev)
    self._ones = torch.ones(self.index.shape[0], dtype=torch.float64, device=dev)

  def update(self, state):
    x = state.reshape(-1).to(torch.float64)
    self.s1.index_add_(0, self.index, x)
    self.s2.index_add_(0, self.index, x * x)
    self.count.index_add_(0, self.index, self._ones)

  def variance(self):
    mean = self.s1 / self.count
    return (self.s2 / self.count - mean * mean).clamp_min(1e-12)

  def inverse_mass(self):
    """The variance as a ragged float32 inverse mass (one entry per element)."""
    return self.variance()[self.index].to(torch.float32)


class MemberDualAveraging:
  """Dual-averaging step-size adaptation (dual_averaging_step_size_adaptation.py:
  353-475) run separately for every member of a batch: each member's accept
  probabilities are reduced with reduce_logmeanexp over its own chains.
  The state is a few float64 scalars per member, updated on the device."""

  def __init__(self, batch, initial_step_size, num_adaptation_steps, target_accept_prob=0.75,
               exploration_shrinkage=0.05, step_count_smoothing=10, decay_rate=0.75):
    dev = _util.device()
    T = len(batch.members)
    s0 = torch.as_tensor(initial_step_size, dtype=torch.float64).reshape(-1).expand(T).to(dev)
    self.batch = batch
    self.n_adapt = int(num_adaptation_steps)
    self.target = float(target_accept_prob)
    self.gamma, self.t0, self.kappa = exploration_shrinkage, step_count_smoothing, decay_rate
    self.log_shrink = torch.log(10.0 * s0)
    self.err = torch.zeros(T, dtype=torch.float64, device=dev)
    self.log_avg = torch.zeros(T, dtype=torch.float64, device=dev)
    self.step = 0
    self.step_size = s0.to(torch.float32).clone()
    self._member = torch.repeat_interleave(torch.arange(T), torch.as_tensor(
        batch.member_chains)).to(dev)
    self._counts = torch.as_tensor(batch.member_chains, dtype=torch.float64, device=dev)

  def update(self, log_accept_ratio):
    lar = torch.nan_to_num(log_accept_ratio.to(torch.float64), nan=-np.inf).clamp(max=0.0)
    T = len(self.batch.members)
    mx = torch.full((T,), -np.inf, dtype=torch.float64, device=lar.device)
    mx = mx.scatter_reduce(0, self._member, lar, 'amax')
    mx = torch.where(torch.isfinite(mx), mx, torch.zeros_like(mx))
    s = torch.zeros(T, dtype=torch.float64, device=lar.device).index_add_(
        0, self._member, torch.exp(lar - mx[self._member]))
    mean_p = torch.exp(torch.log(s) + mx - torch.log(self._counts))
    self.step += 1
    t = float(self.step)
    self.err = self.err + (self.target - mean_p)
    new_log = self.log_shrink - self.err * np.sqrt(t) / ((t + self.t0) * self.gamma)
    eta = t ** -self.kappa
    self.log_avg = eta * new_log + (1 - eta) * self.log_avg
    if self.step < self.n_adapt:
      self.step_size = torch.exp(new_log).to(torch.float32)
    elif self.step == self.n_adapt:
      self.step_size = torch.exp(self.log_avg).to(torch.float32)
    return self.step_size
