#!/usr/bin/env python
"""Throughput of DualAveragingStepSizeAdaptation(NoUTurnSampler) on GB300.

Workload (default, ``nuts_logreg_1e5x100``): Bayesian logistic regression,
X [100000, 100] float32 with column 0 = 1 and the other columns iid
N(0, 1)/sqrt(100), true beta ~ N(0, I), y ~ Bernoulli(sigmoid(X beta)),
prior N(0, I); 1024 chains initialised N(0, 0.1^2); NUTS max_tree_depth=10
inside dual averaging (target accept 0.8, 1000 adaptation steps, initial
step 0.1).  Seeded synthetic data (numpy default_rng(1)).

A step is one transition of the whole 1024-chain batch.  ``value`` is useful
gradient evaluations per second (sum over chains of NUTS leapfrogs_taken,
the reference's accounting, nuts.py:433-435) over the K timed steps with the
chain state resident in HBM.  ``e2e`` repeats K steps through the public
API with the state, log-density and gradients copied in from pinned host
memory and the next state and accept ratios copied back every step.

``--impl reference`` times the CPU restatement of the reference algorithm
(the oracle's samplers in NumPy, the float32 logistic-regression target on
torch CPU ops, all host threads) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# step_size_draws: the step size dual averaging (target 0.8) reaches at the
# end of the 1000-step adaptation window from the Laplace start, in FP32
# (`bench.py --adapt`); the timed transitions are the draws that follow.
WORKLOADS = {
    'nuts_logreg_1e5x100': dict(n=100000, d=100, chains=1024, depth=10, seed=1,
                                feature_scale=0.1, step0=0.1, target_accept=0.8,
                                num_adaptation_steps=1000, precision='fp32', start='laplace',
                                step_size_draws=0.011),
}
# Mixed precision at scale: X 1e6 x 512 BF16, 4096 chains, NUTS depth 8;
# Laplace draws (Newton on the GPU), then --warm-in dual-averaging transitions
# fix the step size of the timed draws.
WORKLOADS['nuts_logreg_1e6x512_bf16'] = dict(n=1000000, d=512, chains=4096, depth=8, seed=2,
                                             feature_scale=512 ** -0.5, step0=0.01,
                                             target_accept=0.8, num_adaptation_steps=1000,
                                             precision='mixed', x_dtype='bf16',
                                             precision_report=10000, start='laplace_da')
WORKLOADS['hmc_logreg_1000x25'] = dict(n=1000, d=25, chains=64, seed=0, feature_scale=1.0,
                                       step0=0.03, leapfrogs=10, burnin=500, precision='fp32')
# Batched uneven posteriors: 128 multivariate normals, D ~ log-U[8, 2048],
# covariance ~ Wishart(D + 2, I / D); 128 non-centred hierarchical normals,
# J ~ U{8..512}, mu ~ N(0, 5^2), tau ~ HalfCauchy(5), sigma_j ~ U(5, 20),
# y_j ~ N(mu + tau z_j, sigma_j^2); 32-512 chains each; NUTS depth 10; one
# step size per posterior from dual averaging during the warm-in.
WORKLOADS['nuts_batch_256'] = dict(mvn=128, hier=128, d_range=(8, 2048), j_range=(8, 512),
                                   chains=(32, 512), depth=10, seed=3, target_accept=0.8)
# Serving: a Poisson(200/s) stream of DA(NUTS) logistic-regression jobs, each
# with N ~ log-U[1e3, 2e5] rows, D ~ log-U[10, 1000] features (BF16 X, N(0,
# 1/D), intercept column), 16-256 chains, 500-5000 draws after 300
# adaptation steps, admitted under a 150 GB device-memory budget.  The timed
# sample is the first `requests` jobs of the stream, at their stated lengths
# and feature counts (above 512 features the mixed target's contractions
# are library GEMMs).
WORKLOADS['serve_logreg_stream'] = dict(rate=200.0, requests=64, length_scale=1.0, seed=4,
                                        n_range=(1e3, 2e5), d_range=(10, 1000),
                                        chains=(16, 256), draws=(500, 5000), adapt=300,
                                        depth=10, budget_gb=150, workers=16)
METRIC = 'grad-evals/s (NUTS leapfrogs_taken summed over chains; min-ESS/s reported beside)'
METRIC_HMC = 'grad-evals/s (HMC: chains x num_leapfrog_steps per transition; min-ESS/s beside)'
METRIC_BATCH = 'grad-evals/s over 256 uneven posteriors in one sampler (sum of min-ESS/s beside)'


def make_data(w):
  rng = np.random.default_rng(w['seed'])
  if w['n'] * w['d'] > 5e7:   # large: draw in float32 directly
    X = rng.standard_normal((w['n'], w['d']), dtype=np.float32)
    X *= np.float32(w['feature_scale'])
  else:
    X = rng.normal(size=(w['n'], w['d'])) * w['feature_scale']
  X[:, 0] = 1.0
  beta = rng.normal(size=w['d'])
  p = 1.0 / (1.0 + np.exp(-(X @ beta.astype(X.dtype))))
  y = (rng.uniform(size=w['n']) < p).astype(np.float32)
  init = (rng.normal(size=(w['chains'], w['d'])) * 0.1).astype(np.float32)
  return X.astype(np.float32), y, init


def engine_features(X, w):
  """X as the engine receives it: BF16 for the BF16-data workloads."""
  import torch
  Xt = torch.from_numpy(X)
  return Xt.to(torch.bfloat16) if w.get('x_dtype') == 'bf16' else Xt


def cpu_gradient_rate(X, y, q, max_seconds):
  """grad-evals/s of the batched log-density + gradient (float32, all host
  threads, see _logreg_f32) on the chains of `q`: the per-leaf cost of NUTS,
  for workloads where one CPU transition would take minutes."""
  target = _logreg_f32(X, y)
  evals = 0
  t0 = time.perf_counter()
  while True:
    target(q)
    evals += q.shape[0]
    if time.perf_counter() - t0 > max_seconds:
      break
  dt = time.perf_counter() - t0
  return evals / dt, evals // q.shape[0], dt


def precision_report(target, X_engine, y, n_states, seed, dev):
  """Engine log-density and gradient against float64 arithmetic on the same
  (BF16) data at n_states random states ~ N(0, I): relative error of the
  log-density and gradient error relative to max |gradient|."""
  import torch
  g = torch.Generator(device=dev)
  g.manual_seed(seed)
  N, D = X_engine.shape
  X64 = X_engine.to(dev).to(torch.float64)
  y64 = torch.as_tensor(y, device=dev, dtype=torch.float64)
  lp_err, g_err = [], []
  chunk, rows = 1000, 100000
  for s0 in range(0, n_states, chunk):
    q = torch.randn(min(chunk, n_states - s0), D, device=dev, generator=g)
    lp, gr = target.log_prob_and_grad(q)
    q64 = q.to(torch.float64)
    lp64 = -0.5 * (q64 * q64).sum(-1) - 0.5 * D * np.log(2 * np.pi)
    g64 = -q64.clone()
    for r0 in range(0, N, rows):
      z = X64[r0:r0 + rows] @ q64.T
      yy = y64[r0:r0 + rows, None]
      lp64 += (yy * z - torch.nn.functional.softplus(z)).sum(0)
      g64 += (yy - torch.sigmoid(z)).T @ X64[r0:r0 + rows]
    lp_err.append(((lp - lp64).abs() / lp64.abs()).cpu())
    g_err.append(((gr.to(torch.float64) - g64).abs().amax(-1) / g64.abs().amax(-1)).cpu())
  lp_err = torch.cat(lp_err)
  g_err = torch.cat(g_err)
  return {'states': n_states, 'reference': 'float64 on the GPU, same BF16 X',
          'log_prob_rel_err_max': float(lp_err.max()), 'log_prob_rel_err_median':
          float(lp_err.median()), 'grad_err_rel_to_max_abs_grad_max': float(g_err.max()),
          'grad_err_rel_to_max_abs_grad_median': float(g_err.median())}


class ClockSampler:
  """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
  FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
            'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
            'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

  def __init__(self, gpu_index):
    self.gpu = gpu_index
    self.proc = None
    self.lines = []

  def start(self):
    try:
      self.proc = subprocess.Popen(
          ['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.FIELDS,
           '--format=csv,noheader,nounits', '-lms', '200'],
          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
      self.thread = threading.Thread(target=self._read, daemon=True)
      self.thread.start()
    except (OSError, ValueError):
      self.proc = None

  def _read(self):
    for line in self.proc.stdout:
      self.lines.append(line.strip())

  def stop(self):
    if self.proc is None:
      return None
    self.proc.terminate()
    try:
      self.proc.wait(timeout=5)
    except subprocess.TimeoutExpired:
      self.proc.kill()
    sm, mx, reasons = [], None, set()
    names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
    for ln in self.lines:
      parts = [p.strip() for p in ln.split(',')]
      if len(parts) < 9:
        continue
      try:
        sm.append(float(parts[1]))
        mx = float(parts[2])
      except ValueError:
        continue
      for nm, v in zip(names, parts[5:9]):
        if v.lower() == 'active':
          reasons.add(nm)
    if not sm:
      return None
    return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': mx, 'reasons': sorted(reasons),
            'samples': len(sm)}


def read_peaks():
  try:
    return json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json'))), 'measured'
  except (OSError, ValueError):
    return {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0, 'bf16_tflops_sustained': 1700.0}, 'fallback'


def read_traffic(workload, kernel_name):
  """Per-launch DRAM traffic (bytes read + written) of the dominant kernel at
  the full chain batch, from the committed ncu summary
  (profiles/traffic.json, keyed 'workload/kernel'), if one was captured."""
  try:
    t = json.load(open(os.path.join(ROOT, 'profiles', 'traffic.json')))
    return t.get('%s/%s' % (workload, kernel_name))
  except (OSError, ValueError):
    return None


def dist_setup(args):
  world = int(os.environ.get('WORLD_SIZE', '1'))
  rank = int(os.environ.get('RANK', '0'))
  local = int(os.environ.get('LOCAL_RANK', '0'))
  return world, rank, local


def cpu_nuts_run(w, X, y, state, eps, keys, max_seconds, timed_from=0):
  """The oracle's DA(NUTS) transitions in the draws phase (step size `eps`,
  adaptation over: dual averaging keeps it) on the host cores: float32 state,
  the float32 logistic-regression target on torch CPU ops with all host
  threads, chains in lock-step as in the reference.  Runs the transitions of
  `keys` (the engine's draws, addressed by chain index, so chains 0..C-1 of
  `state` follow the engine's chains 0..C-1) until `max_seconds` have
  passed; the first `timed_from` are untimed warm-up.  Returns (useful
  gradient evaluations per second, timed transitions, seconds)."""
  from oracle import mcmc as omcmc
  from oracle import philox

  target = _logreg_f32(X, y)
  q = np.array(state, np.float32)
  lp, g = target(q)
  da = omcmc.DualAveraging(eps, w['num_adaptation_steps'], w['target_accept'])
  da.step = w['num_adaptation_steps']                 # adaptation window over
  da.log_averaging_step = np.log(np.float64(eps))
  evals, steps, dt = 0, 0, 0.0
  for i, key in enumerate(keys):
    t0 = time.perf_counter()
    r = omcmc.nuts_one_step(target, q, lp, g, np.float32(da.new_step_size),
                            philox.PhiloxDraws(key), w['depth'], dtype=np.float32)
    q, lp, g = r.next_state, r.target_log_prob, r.grads_target_log_prob
    da.update(r.log_accept_ratio)
    if i >= timed_from:
      dt += time.perf_counter() - t0
      evals += int(r.leapfrogs_taken.sum())
      steps += 1
      if dt > max_seconds:    # the timed budget ends the run (at least one step)
        break
  return evals / max(dt, 1e-9), steps, dt


def _logreg_f32(X, y):
  """The oracle's logistic-regression log-density + gradient in float32 (the
  reference's state type) with an N(0, 1) prior, for the timed CPU legs.
  Evaluated with torch CPU ops on all host threads: the [chains, rows]
  elementwise passes (softplus, sigmoid) dominate, and NumPy runs them on one
  thread, where the reference's compiled CPU path would fuse and parallelise
  them (5-6x slower at 1e5 x 100 x 1024 on 8 cores)."""
  import torch
  torch.set_num_threads(os.cpu_count() or 1)
  Xt = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32))
  yt = torch.from_numpy(np.ascontiguousarray(y, dtype=np.float32))
  half_log_2pi = 0.5 * np.log(2 * np.pi)

  def target(q):
    qt = torch.from_numpy(np.ascontiguousarray(q, dtype=np.float32))
    z = qt @ Xt.T                                                # [C, N]
    sp = torch.nn.functional.softplus(z)
    lp = (yt * z - sp).sum(-1, dtype=torch.float64)              # bernoulli.py:126-140
    lp += (-0.5 * qt.double() ** 2 - half_log_2pi).sum(-1)
    g = (yt - torch.sigmoid(z)) @ Xt - qt
    return lp.numpy(), g.numpy()
  return target


def cpu_hmc_run(w, X, y, init, max_seconds, warmup, steps):
  """Time the oracle's HMC + Metropolis-Hastings transition (hmc.py:661-875,
  metropolis_hastings.py:160-254; float32, all host threads) on every chain:
  `warmup` untimed transitions, then up to `steps` timed ones (at least one)
  within `max_seconds`.  Transition t uses sample_chain's key t, so a
  fixed-step HMC run costs the same per transition from any state."""
  from oracle import mcmc as omcmc
  from oracle import philox
  target = _logreg_f32(X, y)
  q = init.copy()
  lp, g = target(q)
  evals, done, dt = 0, 0, 0.0
  for t in range(warmup + steps):
    t0 = time.perf_counter()
    r = omcmc.hmc_one_step(target, q, lp, g, np.float32(w['step0']), w['leapfrogs'],
                           philox.PhiloxDraws(philox.step_key((w['seed'], 0), t)),
                           dtype=np.float32)
    q, lp, g = r.next_state, r.target_log_prob, r.grads_target_log_prob
    if t >= warmup:
      dt += time.perf_counter() - t0
      evals += q.shape[0] * w['leapfrogs']
      done += 1
      if dt > max_seconds:
        break
  return evals / max(dt, 1e-9), done, dt


def run_reference(args, w):
  """--impl reference: the CPU restatement of the reference algorithms (the
  oracle; TensorFlow Probability itself cannot be installed here) on the host
  cores, for the workload, metric and unit of the engine's line."""
  world, rank, _ = dist_setup(args)
  if rank != 0:
    return
  budget = float(os.environ.get('GBM_REFERENCE_SECONDS', '300'))
  cores = os.cpu_count()
  par = 'single' if world == 1 else 'rank 0 only (host cores)'
  if args.workload.startswith('serve_'):
    print(json.dumps({'impl': 'reference', 'unavailable':
                      'the serving workload measures a job server over a request stream; the '
                      'reference has no server (its per-job sampler cost is the nuts_logreg '
                      'reference arm)'}), flush=True)
    return
  if args.workload.startswith('nuts_batch'):
    spec = make_batch_members(w)
    rate, passes, dt, pick = cpu_batch_gradient_rate(spec, min(budget, 60.0))
    metric, steps = METRIC_BATCH, passes
    config = {'workload': args.workload, 'posteriors': len(spec),
              'max_tree_depth': w['depth'], 'precision': 'f64 (NumPy oracle targets)',
              'parallelism': par}
    sample = ('%d passes of the log-prob+gradient of %d of the %d posteriors with all their '
              'chains (%.1f s; the NUTS leaf cost, no tree bookkeeping); NumPy float64 oracle '
              'targets, BLAS threads = %d' % (passes, len(pick), len(spec), dt, cores))
  elif args.workload.startswith('hmc_'):
    X, y, init = make_data(w)
    rate, steps, dt = cpu_hmc_run(w, X, y, init, budget, args.warmup, args.steps)
    metric = METRIC_HMC
    config = hmc_config(args, w, 'fp32')
    sample = ('each step: one HMC transition (10 leapfrog steps) of all %d chains, after %d '
              'untimed warm-up transitions (a fixed-step HMC transition costs the same from '
              'any state); oracle HMC + Metropolis-Hastings in NumPy, float32 target on torch '
              'CPU ops, %d threads; %d of %d timed steps (%.2f s timed)'
              % (w['chains'], args.warmup, cores, steps, args.steps, dt))
  else:
    X, y, init = make_data(w)
    metric = METRIC
    config = {'workload': args.workload, 'rows': w['n'], 'features': w['d'],
              'chains': w['chains'], 'max_tree_depth': w['depth'],
              'target_accept_prob': w.get('target_accept'),
              'num_adaptation_steps': w.get('num_adaptation_steps'),
              'precision': 'fp32 (NumPy oracle)', 'parallelism': par}
    if w['n'] * w['d'] > 5e7:
      # One CPU transition of this size would take hours: time the NUTS leaf
      # cost (batched log-prob + gradient) of a 64-chain sample instead.
      sub = min(64, w['chains'])
      rate, steps, dt = cpu_gradient_rate(X, y, init[:sub], min(budget, 60.0))
      sample = ('%d batched log-prob+gradient evaluations of %d of the %d chains (%.1f s; the '
                'NUTS leaf cost, no tree bookkeeping); float32 torch CPU ops, %d threads'
                % (steps, sub, w['chains'], dt, cores))
    else:
      from oracle import philox
      # The engine arm's timed transitions: same Laplace start, step size and
      # keys (sample_chain steps num_adaptation_steps + i), all chains; the
      # first `warmup` transitions are run untimed, as in the engine arm.
      init = laplace_start(X, y, w['chains'], w['seed'])
      sub = min(int(os.environ.get('GBM_REFERENCE_CHAINS', '128')), w['chains'])
      t0 = w['num_adaptation_steps']
      keys = [philox.step_key((w['seed'], 0), t0 + i) for i in range(args.warmup + args.steps)]
      rate, steps, dt = cpu_nuts_run(w, X, y, init[:sub], w['step_size_draws'], keys, budget,
                                     timed_from=args.warmup)
      config = nuts_config(args, w, 'fp32', world)
      sample = ('each step: one DA(NUTS) transition of chains 0-%d of the %d, in the draws '
                'phase, from the same Laplace start, step size %g and transition keys as the '
                'engine arm, so these chains follow the engine\'s chains 0-%d (same draws); %d '
                'untimed warm-up transitions first; oracle NUTS in NumPy (chains in lock-step), '
                'float32 target on torch CPU ops, %d threads; %d of %d timed steps within the '
                '%.0f s budget (%.1f s timed)'
                % (sub - 1, w['chains'], w['step_size_draws'], sub - 1, args.warmup, cores,
                   steps, args.steps, budget, dt))
  line = {
      'impl': 'reference', 'metric': metric, 'value': rate, 'unit': 'grad-evals/s',
      'n_gpus': args.gpus, 'steps': steps,
      'warmup': args.warmup if (w.get('start') == 'laplace' or
                                args.workload.startswith('hmc_')) else 0,
      'ms_per_step': 1000 * dt / max(steps, 1),
      'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
      'data': ('synthetic (seeded numpy default_rng(%d))' % w['seed']) if 'seed' in w
              else 'synthetic (seeded numpy)', 'config': config,
      'cpu_baseline': {'value': rate, 'unit': 'grad-evals/s', 'cores': cores, 'kind': 'port',
                       'sample': sample},
      'e2e': {'value': rate, 'unit': 'grad-evals/s', 'h2d_bytes_per_step': 0,
              'd2h_bytes_per_step': 0},
  }
  print(json.dumps(line), flush=True)


def run_kernel_only(args, w):
  """Time the batched gradient alone at the full chain batch (profiling aid)."""
  import torch
  import probability_gb300 as pg
  if args.kernel_rows:   # a smaller case of the same shape (profiling)
    w = dict(w, n=args.kernel_rows)
  if args.kernel_shape:   # rows,features,chains of another logistic posterior
    n, d, c = (int(v) for v in args.kernel_shape.split(','))
    w = dict(w, n=n, d=d, chains=c, feature_scale=d ** -0.5)
  X, y, init = make_data(w)
  target = pg.LogisticRegression(engine_features(X, w), y,
                                 precision=args.precision or w['precision'])
  q = torch.from_numpy(init).cuda()
  for _ in range(args.warmup):
    target.log_prob_and_grad(q)
  torch.cuda.synchronize()
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  e0.record()
  for _ in range(args.steps):
    target.log_prob_and_grad(q)
  e1.record()
  e1.synchronize()
  ms = e0.elapsed_time(e1) / args.steps
  flops, nbytes = target.cost(q.shape[0])
  print(json.dumps({'kernel_only': True, 'precision': target.precision, 'ms_per_eval': ms,
                    'tflops': flops / ms / 1e9, 'chains': q.shape[0]}), flush=True)


def hmc_config(args, w, precision):
  return {'workload': args.workload, 'rows': w['n'], 'features': w['d'],
          'chains': w['chains'], 'step_size': w['step0'],
          'num_leapfrog_steps': w['leapfrogs'], 'burnin': w['burnin'],
          'precision': precision, 'l2': 'inputs L2-resident (100 KB of X)',
          'parallelism': 'single'}


def run_hmc(args, w):
  """HMC on the 1000 x 25 logistic regression (64 chains, step 0.03, 10
  leapfrog steps): burn-in untimed, then K transitions timed through the
  device-resident chain loop (one CUDA graph per transition)."""
  import torch
  import probability_gb300 as pg
  X, y, init = make_data(w)
  precision = args.precision or w['precision']
  target = pg.LogisticRegression(X, y, precision=precision)
  k = pg.mcmc.HamiltonianMonteCarlo(target, step_size=w['step0'],
                                    num_leapfrog_steps=w['leapfrogs'])
  q = torch.from_numpy(init).cuda()
  run = pg.mcmc.run_chain(k, 1, q, num_burnin_steps=w['burnin'] + args.warmup - 1,
                          seed=(w['seed'], 0))
  q = run.final_state
  first = w['burnin'] + args.warmup
  clocks = ClockSampler(torch.cuda.current_device())
  clocks.start()
  torch.cuda.synchronize()
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  e0.record()
  run = pg.mcmc.run_chain(k, args.steps, q, seed=(w['seed'], 0), first_step=first)
  e1.record()
  e1.synchronize()
  clk = clocks.stop()
  secs = e0.elapsed_time(e1) / 1000.0
  evals = args.steps * w['chains'] * w['leapfrogs']
  acc = run.trace['is_accepted'].float().mean().item()
  # ESS per draw from 500 further (untimed) draws of the same chains: the
  # timed window is too short for a stable autocorrelation estimate.
  n_ess = 500
  ess_run = pg.mcmc.run_chain(k, n_ess, run.final_state, seed=(w['seed'], 0),
                              first_step=first + args.steps)
  ess = pg.mcmc.effective_sample_size(ess_run.all_states, filter_beyond_positive_pairs=True,
                                      cross_chain_dims=1)
  ess_per_draw = float(ess.min().item()) / n_ess

  # ---- end to end: HamiltonianMonteCarlo.one_step with host buffers ----
  C, D = q.shape
  h_state = torch.from_numpy(init).pin_memory()
  kr = k.bootstrap_results(torch.from_numpy(init).cuda())
  h_tlp = kr.accepted_results.target_log_prob.cpu().pin_memory()
  h_grad = kr.accepted_results.grads_target_log_prob.cpu().pin_memory()
  h_out = torch.empty((C, D), dtype=torch.float32).pin_memory()
  h_acc = torch.empty(C, dtype=torch.bool).pin_memory()
  for t in range(args.warmup + args.steps):
    if t == args.warmup:
      torch.cuda.synchronize()
      e0.record()
    acc_r = kr.accepted_results._replace(
        target_log_prob=h_tlp.cuda(non_blocking=True),
        grads_target_log_prob=h_grad.cuda(non_blocking=True))
    s_, kr = k.one_step(h_state.cuda(non_blocking=True), kr._replace(accepted_results=acc_r),
                        seed=pg._util.step_key((w['seed'], 0), t))
    h_out.copy_(s_, non_blocking=True)
    h_tlp.copy_(kr.accepted_results.target_log_prob, non_blocking=True)
    h_grad.copy_(kr.accepted_results.grads_target_log_prob, non_blocking=True)
    h_acc.copy_(kr.is_accepted, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    h_state.copy_(h_out)
  e1.record()
  e1.synchronize()
  e2e_s = e0.elapsed_time(e1) / 1000.0
  e2e = {'value': evals / e2e_s, 'unit': 'grad-evals/s',
         'h2d_bytes_per_step': C * D * 4 * 2 + C * 8, 'd2h_bytes_per_step': C * D * 8 + C * 9,
         'steps': args.steps,
         'transitions': 'HamiltonianMonteCarlo.one_step per transition, state, log-density and '
                        'gradients copied in from pinned host memory and back every step'}

  # ---- roofline: the batched gradient alone at the 64-chain batch ----
  reps = 200
  for _ in range(10):
    target.log_prob_and_grad(q)
  e0.record()
  for _ in range(reps):
    target.log_prob_and_grad(q)
  e1.record()
  e1.synchronize()
  t_eval = e0.elapsed_time(e1) / 1000.0 / reps
  flops, _ = target.cost(C)
  peaks, _ = read_peaks()
  sm_max = (clk or {}).get('sm_max_mhz') or peaks.get('sm_max_mhz', 2070.0)
  peak, sms = fp32_peak_tflops(sm_max)
  achieved = flops / t_eval / 1e12
  roofline = {'bound': 'fp32', 'achieved': achieved, 'peak': peak, 'unit': 'TFLOP/s',
              'frac': achieved / peak, 'traffic': read_traffic(args.workload,
                                                               kernel_name(precision, D)),
              'kernel': kernel_name(precision, D),
              'peak_source': 'nominal FP32 FMA rate: %d SMs x 128 lanes x 2 flop x %.0f MHz'
                             % (sms, sm_max),
              'eval_us': 1e6 * t_eval,
              'note': 'X is 100 KB and the batch 64 chains: one evaluation is a few '
                      'microseconds of latency (launch + one row split per CTA), far from '
                      'any throughput roof; the bound that matters here is latency'}
  cpu = None
  if not args.no_cpu_baseline:
    budget = float(os.environ.get('GBM_CPU_BASELINE_SECONDS', '20'))
    rate, nsteps, dt = cpu_hmc_run(w, X, y, init, budget, args.warmup, args.steps)
    cpu = {'value': rate, 'unit': 'grad-evals/s', 'cores': os.cpu_count(), 'kind': 'port',
           'sample': '%d HMC transitions of all %d chains after %d untimed (%.2f s); oracle '
                     'HMC + Metropolis-Hastings in NumPy, float32 target on torch CPU ops, '
                     'all host threads' % (nsteps, C, args.warmup, dt)}
  print(json.dumps({
      'metric': METRIC_HMC, 'value': evals / secs, 'unit': 'grad-evals/s', 'n_gpus': 1,
      'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1000 * secs / args.steps,
      'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
      'data': 'synthetic (seeded numpy default_rng(0))',
      'config': hmc_config(args, w, precision),
      'min_ess_per_s': ess_per_draw * args.steps / secs,
      'min_ess_note': 'min over dimensions of cross-chain ESS (diagnostic.py:203-337) of 500 '
                      'further draws, per draw, times the timed draws per second',
      'accept_rate': acc, 'e2e': e2e, 'roofline': roofline, 'cpu_baseline': cpu,
      # per transition: momentum + half kick, L x (gradient kernel + split
      # reduction), L - 1 kick-drift, MH finish, next step key
      'gpu_launches': args.steps * (3 * w['leapfrogs'] + 2),
      'clocks': clk}), flush=True)


def laplace_start(X, y, chains, seed, prior_scale=1.0, iters=25):
  """Chain states drawn from the posterior's Laplace approximation
  N(beta_MAP, H^-1), H = X^T diag(s(1 - s)) X + I / prior_scale^2, with
  beta_MAP from Newton's method (float64 NumPy, seeded): a start in the
  typical set, shared by the engine and the reference arm, so that both time
  transitions of the same (stationary) regime from the same state."""
  X64 = np.asarray(X, np.float64)
  y64 = np.asarray(y, np.float64)
  D = X64.shape[1]
  prec = 1.0 / prior_scale ** 2
  beta = np.zeros(D)
  for _ in range(iters):
    z = X64 @ beta
    s = 1.0 / (1.0 + np.exp(-z))
    g = X64.T @ (y64 - s) - prec * beta
    H = (X64 * (s * (1.0 - s))[:, None]).T @ X64 + prec * np.eye(D)
    step = np.linalg.solve(H, g)
    beta = beta + step
    if np.max(np.abs(step)) < 1e-12:
      break
  s = 1.0 / (1.0 + np.exp(-(X64 @ beta)))
  H = (X64 * (s * (1.0 - s))[:, None]).T @ X64 + prec * np.eye(D)
  L = np.linalg.cholesky(H)
  zz = np.random.default_rng(seed + 100).standard_normal((chains, D))
  draws = beta + np.linalg.solve(L.T, zz.T).T            # cov = H^-1
  return draws.astype(np.float32)


def laplace_start_device(X_engine, y, chains, seed, dev, prior_scale=1.0, iters=30):
  """laplace_start on the GPU in float64 (torch), for data too large for a
  host Newton solve: the MAP by Newton's method on the engine's X (BF16
  values where the workload stores BF16), then N(beta_MAP, H^-1) draws from
  a seeded NumPy generator."""
  import torch
  X = X_engine.to(dev).to(torch.float64)
  yv = torch.as_tensor(y, dtype=torch.float64, device=dev)
  D = X.shape[1]
  prec = 1.0 / prior_scale ** 2
  eye = torch.eye(D, dtype=torch.float64, device=dev)
  beta = torch.zeros(D, dtype=torch.float64, device=dev)

  def hessian(b):
    s = torch.sigmoid(X @ b)
    return (X * (s * (1.0 - s))[:, None]).T @ X + prec * eye, s

  for _ in range(iters):
    H, s = hessian(beta)
    g = X.T @ (yv - s) - prec * beta
    step = torch.linalg.solve(H, g)
    beta = beta + step
    if float(step.abs().max()) < 1e-12:
      break
  H, _ = hessian(beta)
  L = torch.linalg.cholesky(H)
  zz = torch.from_numpy(np.random.default_rng(seed + 100).standard_normal((chains, D))).to(dev)
  draws = beta + torch.linalg.solve_triangular(L.T, zz.T, upper=True).T   # cov = H^-1
  del X
  return draws.to(torch.float32).cpu().numpy()


def draws_phase_keys(w, count):
  """Keys of the timed transitions: sample_chain's per-step keys (seed, 0)
  at steps num_adaptation_steps, num_adaptation_steps + 1, ... (the first
  draws after adaptation)."""
  from probability_gb300 import _util
  t0 = w['num_adaptation_steps']
  return [_util.step_key((w['seed'], 0), t0 + i) for i in range(count)]


def post_adaptation_results(kernel, state, eps, dev):
  """DualAveragingStepSizeAdaptation results after its adaptation window:
  step == num_adaptation_steps, so every later transition keeps `eps`
  (dual_averaging_step_size_adaptation.py:468-474)."""
  import torch
  kr = kernel.bootstrap_results(state)
  e = torch.full_like(kr.new_step_size, eps)
  return kr._replace(step=int(kernel.num_adaptation_steps),
                     log_averaging_step=torch.log(e.to(torch.float64)), new_step_size=e)


def fp32_peak_tflops(sm_max_mhz):
  """Nominal FP32 rate of the CUDA cores: SMs x 128 FMA lanes x 2 flop x the
  maximum SM clock (the FP32 form's roof; MEASURED_PEAKS.json holds the HBM
  and BF16 tensor peaks only)."""
  import torch
  sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
  return sms * 128 * 2 * sm_max_mhz * 1e6 / 1e12, sms


class Leg:
  """Timed DA(NUTS) transitions of one target precision from one start."""

  def __init__(self, pg, X_engine, y, w, precision, eps, dev):
    self.pg = pg
    self.target = pg.LogisticRegression(X_engine, y, precision=precision)
    self.nuts = pg.mcmc.NoUTurnSampler(self.target, step_size=eps, max_tree_depth=w['depth'])
    self.kernel = pg.mcmc.DualAveragingStepSizeAdaptation(
        self.nuts, num_adaptation_steps=w['num_adaptation_steps'],
        target_accept_prob=w['target_accept'])
    self.eps, self.dev = eps, dev

  def start(self, state):
    return state.clone(), post_adaptation_results(self.kernel, state, self.eps, self.dev)

  def prewarm(self, state, n, seed):
    """Transitions from a copy of `state` with unrelated keys, discarded:
    they capture the per-depth leaf graphs outside the timed region."""
    q, kr = self.start(state)
    for i in range(n):
      q, kr = self.kernel.one_step(q, kr, seed=self.pg._util.step_key(seed, 10 ** 6 + i))
    import torch
    torch.cuda.synchronize()

  def run(self, q, kr, keys, l2_flush=None, timed=True):
    """Transitions with `keys`; with timed, CUDA events on the launching
    stream bracket each one (L2 flushed outside the events)."""
    import torch
    step_ms, wall_s = [], []
    lf = torch.zeros((), dtype=torch.int64, device=self.dev)
    draws = []
    for key in keys:
      if l2_flush is not None:
        l2_flush.zero_()
      if timed:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        e0.record()
      q, kr = self.kernel.one_step(q, kr, seed=key)
      if timed:
        e1.record()
        e1.synchronize()
        wall_s.append(time.perf_counter() - w0)
        step_ms.append(e0.elapsed_time(e1))
      lf += kr.inner_results.leapfrogs_taken.sum()
      draws.append(q)
    return q, kr, dict(step_ms=step_ms, wall_s=wall_s, lf=int(lf.item()), draws=draws)

  def profiled(self, q, kr, keys):
    """The same transitions with CUDA events around every batched gradient
    (leaf-by-leaf launches): device time of the gradient kernels."""
    import ctypes
    _native = self.pg._native
    h = self.nuts._handle
    z = (ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64())
    _native.check(_native.lib().gbm_nuts_read_profile(h, *map(ctypes.byref, z)))
    _native.check(_native.lib().gbm_nuts_set_profiling(h, 1))
    leaves = 0
    import torch
    lf = torch.zeros((), dtype=torch.int64, device=self.dev)
    for key in keys:
      q, kr = self.kernel.one_step(q, kr, seed=key)
      leaves += int(getattr(self.nuts, 'last_leaf_iterations', 0) or 0)
      lf += kr.inner_results.leapfrogs_taken.sum()
    ms, ev, la = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
    _native.check(_native.lib().gbm_nuts_read_profile(h, ctypes.byref(ms), ctypes.byref(ev),
                                                      ctypes.byref(la)))
    _native.lib().gbm_nuts_set_profiling(h, 0)
    return q, kr, dict(eval_ms=ms.value, evals=int(ev.value), leaves=leaves, lf=int(lf.item()))

  def launches(self):
    import ctypes
    _native = self.pg._native
    z = (ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64())
    _native.check(_native.lib().gbm_nuts_read_profile(self.nuts._handle, *map(ctypes.byref, z)))
    return int(z[2].value)


def kernel_name(precision, d):
  if precision == 'fp32':
    return 'logreg_f32_kernel' if d <= 128 else 'logreg_partial_kernel'
  return ('logreg_tc_pair_kernel' if d > 256 else 'logreg_tc_kernel' if d > 128 else
          'logreg_tct_kernel')


def leg_roofline(leg, prof, workload, d, sm_max_mhz, measured_over):
  """Roofline of the dominant kernel (the batched gradient: partial kernel
  + split reduction) from the profiled pass: algorithmic 4 N D flops per
  useful gradient evaluation over the summed event time of the launches."""
  flops_per_grad, _ = leg.target.cost(1)
  eval_s = prof['eval_ms'] / 1000.0
  achieved = flops_per_grad * prof['lf'] / eval_s / 1e12 if eval_s > 0 else None
  name = kernel_name(leg.target.precision, d)
  if leg.target.precision == 'fp32':
    peak, sms = fp32_peak_tflops(sm_max_mhz)
    bound, src = 'fp32', ('nominal FP32 FMA rate: %d SMs x 128 lanes x 2 flop x %.0f MHz '
                          '(MEASURED_PEAKS.json has no FP32 CUDA-core peak)' % (sms, sm_max_mhz))
  else:
    peaks, peak_src = read_peaks()
    peak, bound = peaks['bf16_tflops'], 'tensor'
    src = peak_src + ' (MEASURED_PEAKS.json bf16_tflops burst)'
  return {'bound': bound, 'achieved': achieved, 'peak': peak, 'unit': 'TFLOP/s',
          'frac': achieved / peak if achieved else None,
          'traffic': read_traffic(workload, name), 'kernel': name, 'peak_source': src,
          'eval_launches': prof['evals'], 'eval_ms_total': prof['eval_ms'],
          'alg_flops_per_grad_eval': flops_per_grad, 'measured_over': measured_over}


def min_ess_per_s(pg, draws, secs):
  """min over dimensions of the cross-chain ESS (diagnostic.py:220-275, with
  filter_beyond_positive_pairs) of the timed draws, per second."""
  import torch
  if len(draws) < 4:
    return None
  ess = pg.mcmc.effective_sample_size(torch.stack(draws), filter_beyond_positive_pairs=True,
                                      cross_chain_dims=1)
  return float(ess.min().item()) / secs


def split_rhat_max(pg, draws):
  import torch
  if len(draws) < 4:
    return None
  try:
    return float(pg.mcmc.potential_scale_reduction(torch.stack(draws),
                                                   split_chains=True).max().item())
  except Exception:   # a diagnostic must never fail the benchmark line
    return None


def nuts_config(args, w, precision, world=1, eps=None):
  start = w.get('start')
  if start == 'laplace':
    desc = ('Laplace approximation of the posterior (seeded), step size %g: the draws phase '
            'after adaptation' % w['step_size_draws'])
  elif start == 'laplace_da':
    desc = ('Laplace approximation of the posterior (seeded, Newton on the GPU in float64), '
            'then %d dual-averaging transitions; the timed transitions keep step size %s '
            '(geometric mean of the second half), the draws phase after adaptation'
            % (args.warm_in, '%.6g' % eps if eps else 'from the warm-in'))
  else:
    desc = '%d dual-averaging warm-in transitions from N(0, 0.1^2)' % args.warm_in
  laplace = start in ('laplace', 'laplace_da')
  return {'workload': args.workload, 'rows': w['n'], 'features': w['d'],
          'chains': w['chains'], 'max_tree_depth': w['depth'],
          'target_accept_prob': w['target_accept'],
          'num_adaptation_steps': w['num_adaptation_steps'],
          'precision': precision, 'start': desc,
          'timed_transitions': 'keys of sample_chain steps %d.. (after %d warm-up steps)'
                               % (w['num_adaptation_steps'] + args.warmup, args.warmup)
                               if laplace else 'after the warm-in',
          'l2': 'flushed between timed steps (256 MB write outside the step events)',
          'parallelism': 'single' if world == 1 else 'replicas x %d' % world}


def run_engine(args, w):
  import torch
  world, rank, local = dist_setup(args)
  torch.cuda.set_device(local)
  dist = None
  if world > 1:
    import torch.distributed as dist
    dist.init_process_group('nccl')
  import probability_gb300 as pg
  from probability_gb300 import replicas
  dev = torch.device('cuda', local)
  X, y, init = make_data(w)
  laplace = w.get('start') in ('laplace', 'laplace_da')
  X_engine = engine_features(X, w)
  if laplace:
    start_seed = w['seed'] + 7919 * rank
    init = laplace_start(X, y, w['chains'], start_seed) if w['start'] == 'laplace' else \
        laplace_start_device(X_engine, y, w['chains'], start_seed, dev)
  elif world > 1:  # independent replicas: per-rank initial state
    init = replicas.replica_init(init.shape, w['seed'], rank)
  precision = args.precision or w['precision']
  state0 = torch.from_numpy(init).to(dev)
  l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
  peaks, _ = read_peaks()

  def barrier():
    if dist is not None:
      dist.barrier()
    torch.cuda.synchronize()

  def keys_for(count, offset=0):
    if laplace:
      ks = draws_phase_keys(w, offset + count)[offset:]
    else:
      ks = [pg._util.step_key((w['seed'], 0), args.warm_in + offset + i) for i in range(count)]
    if world > 1:
      ks = [replicas.replica_key(k, rank) for k in ks]
    return ks

  if laplace:
    eps = w.get('step_size_draws')
    if w['start'] == 'laplace_da':
      # Dual averaging from the Laplace draws; the timed transitions keep the
      # geometric mean of the step sizes of its second half.
      warm = Leg(pg, X_engine, y, w, precision, w['step0'], dev)
      q = state0.clone()
      kr = warm.kernel.bootstrap_results(q)
      logs = []
      for i in range(args.warm_in):
        q, kr = warm.kernel.one_step(q, kr, seed=pg._util.step_key((w['seed'], 2), i))
        if i >= args.warm_in // 2:
          logs.append(float(torch.log(kr.new_step_size.reshape(-1)[0]).item()))
      eps = float(np.exp(np.mean(logs)))
      state0 = q
      del warm, kr
    leg = Leg(pg, X_engine, y, w, precision, eps, dev)
    leg.prewarm(state0, args.prewarm, (w['seed'], 1))
    q, kr = leg.start(state0)
  else:
    # Dual-averaging warm-in from N(0, 0.1^2) (adaptation still running).
    leg = Leg(pg, X_engine, y, w, precision, w['step0'], dev)
    q = state0.clone()
    kr = leg.kernel.bootstrap_results(q)
    for i in range(args.warm_in):
      q, kr = leg.kernel.one_step(q, kr, seed=pg._util.step_key((w['seed'], 0), i))
    eps = float(kr.new_step_size.reshape(-1)[0].item())
  start_q, start_kr = q.clone(), kr
  q, kr, _ = leg.run(q, kr, keys_for(args.warmup), timed=False)
  la0 = leg.launches()
  clocks = ClockSampler(local)
  clocks.start()
  barrier()
  q, kr, tm = leg.run(q, kr, keys_for(args.steps, args.warmup), l2_flush=l2_flush)
  barrier()
  clk = clocks.stop()
  launches = leg.launches() + args.steps     # + one DA update per step
  del la0
  secs = sum(tm['step_ms']) / 1000.0
  secs, grad_evals = replicas.combine_throughput(secs, tm['lf'])   # max time, total work
  value = grad_evals / secs
  ess_s = min_ess_per_s(pg, tm['draws'], sum(tm['step_ms']) / 1000.0)
  rhat = split_rhat_max(pg, tm['draws'])
  sm_max = (clk or {}).get('sm_max_mhz') or peaks.get('sm_max_mhz', 2070.0)
  # Profiled pass: the next K transitions, leaf by leaf with events.
  q, kr, prof = leg.profiled(q, kr, keys_for(args.steps, args.warmup + args.steps))
  roofline = leg_roofline(leg, prof, args.workload, w['d'], sm_max,
                          'a profiled pass of %d further transitions (events around every '
                          'batched gradient; the timed region replays graphs)' % args.steps)

  # ---- end-to-end through host buffers (public API, pinned memory) ----
  C, D = q.shape
  h_state = torch.empty((C, D), dtype=torch.float32).pin_memory()
  h_tlp = torch.empty(C, dtype=torch.float64).pin_memory()
  h_grad = torch.empty((C, D), dtype=torch.float32).pin_memory()
  h_out = torch.empty((C, D), dtype=torch.float32).pin_memory()
  h_lar = torch.empty(C, dtype=torch.float64).pin_memory()
  h_state.copy_(start_q.cpu())
  h_tlp.copy_(start_kr.inner_results.target_log_prob.cpu())
  h_grad.copy_(start_kr.inner_results.grads_target_log_prob.cpu())
  kr = start_kr
  e2e_keys = keys_for(args.warmup + args.steps)[args.warmup:]
  if laplace:   # the same transitions again, from the host-resident start
    q_, kr_, _ = leg.run(start_q.clone(), start_kr, keys_for(args.warmup), timed=False)
    h_state.copy_(q_.cpu())
    h_tlp.copy_(kr_.inner_results.target_log_prob.cpu())
    h_grad.copy_(kr_.inner_results.grads_target_log_prob.cpu())
    kr = kr_
  lf_e2e = torch.zeros((), dtype=torch.int64, device=dev)
  barrier()
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  e0.record()
  for key in e2e_keys:
    d_state = h_state.to(dev, non_blocking=True)
    inner = kr.inner_results._replace(
        target_log_prob=h_tlp.to(dev, non_blocking=True),
        grads_target_log_prob=h_grad.to(dev, non_blocking=True))
    kr = kr._replace(inner_results=inner)
    s_, kr = leg.kernel.one_step(d_state, kr, seed=key)
    lf_e2e += kr.inner_results.leapfrogs_taken.sum()
    h_out.copy_(s_, non_blocking=True)
    h_lar.copy_(kr.inner_results.log_accept_ratio, non_blocking=True)
    h_tlp.copy_(kr.inner_results.target_log_prob, non_blocking=True)
    h_grad.copy_(kr.inner_results.grads_target_log_prob, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    h_state.copy_(h_out)
  e1.record()
  e1.synchronize()
  e2e_s = e0.elapsed_time(e1) / 1000.0
  e2e_value = int(lf_e2e.item()) / e2e_s
  h2d = C * D * 4 * 2 + C * 8
  d2h = C * D * 4 * 2 + C * 8 * 2

  # ---- the other precision on the same GPU, same start and transitions ----
  other = None
  other_prec = 'mixed' if precision == 'fp32' else 'fp32'
  # (The FP32 form of the 1e6 x 512 workload would need the library-GEMM
  # target's N x chains buffers, tens of GB: only the stated arithmetic runs.)
  if args.other_precision and w['n'] * w['d'] <= 5e7:
    X_other = X if other_prec == 'fp32' else X_engine
    leg2 = Leg(pg, X_other, y, w, other_prec, eps, dev)
    leg2.prewarm(state0, args.prewarm, (w['seed'], 1))
    q2, kr2 = leg2.start(start_q)
    kr2 = kr2._replace(inner_results=kr2.inner_results)
    q2, kr2, _ = leg2.run(q2, kr2, keys_for(args.warmup), timed=False)
    barrier()
    q2, kr2, tm2 = leg2.run(q2, kr2, keys_for(args.steps, args.warmup), l2_flush=l2_flush)
    secs2 = sum(tm2['step_ms']) / 1000.0
    q2, kr2, prof2 = leg2.profiled(q2, kr2, keys_for(args.steps, args.warmup + args.steps))
    ess2 = min_ess_per_s(pg, tm2['draws'], secs2)
    other = {'precision': other_prec, 'value': tm2['lf'] / secs2, 'unit': 'grad-evals/s',
             'ms_per_step': 1000 * secs2 / args.steps, 'min_ess_per_s': ess2,
             'roofline': leg_roofline(leg2, prof2, args.workload, w['d'], sm_max,
                                      'a profiled pass of %d further transitions'
                                      % args.steps),
             'note': 'same start state, step size and transition keys as the main line'}
    if precision == 'fp32':
      other['speedup_vs_fp32_grad_evals'] = other['value'] / value
      other['speedup_vs_fp32_min_ess_per_s'] = (ess2 / ess_s) if ess2 and ess_s else None
    del leg2

  cpu = None
  if rank == 0 and world == 1 and not args.no_cpu_baseline and w['n'] * w['d'] > 5e7:
    budget = float(os.environ.get('GBM_CPU_BASELINE_SECONDS', '20'))
    sub = 64
    rate, nev, dt = cpu_gradient_rate(X, y, start_q[:sub].cpu().numpy(), budget)
    cpu = {'value': rate, 'unit': 'grad-evals/s', 'cores': os.cpu_count(), 'kind': 'port',
           'sample': '%d batched log-prob+gradient evaluations of %d of the %d chains '
                     '(%.1f s; the NUTS leaf cost, no tree bookkeeping); float32 torch '
                     'CPU ops, all host threads' % (nev, sub, w['chains'], dt)}
  elif rank == 0 and world == 1 and not args.no_cpu_baseline:
    budget = float(os.environ.get('GBM_CPU_BASELINE_SECONDS', '20'))
    sub = 64
    rate, nsteps, dt = cpu_nuts_run(w, X, y, init[:sub], eps, keys_for(10 ** 4), budget)
    cpu = {'value': rate, 'unit': 'grad-evals/s', 'cores': os.cpu_count(), 'kind': 'port',
           'sample': '%d NUTS transitions of chains 0-%d of %d (%.1f s), from the same start, '
                     'step size and transition keys as the timed region (the same draws); '
                     'oracle NUTS in NumPy (chains in lock-step as in the reference), float32 '
                     'target on torch CPU ops, all host threads'
                     % (nsteps, sub - 1, w['chains'], dt)}

  prec_report = None
  if rank == 0 and w.get('precision_report'):
    prec_report = precision_report(leg.target, X_engine, y, w['precision_report'], w['seed'],
                                   dev)

  if rank == 0:
    wall = sum(tm['wall_s'])
    line = {
        'metric': METRIC, 'value': value, 'unit': 'grad-evals/s', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1000 * secs / args.steps,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32' if precision == 'fp32' else 'bf16+f32',
        'data': 'synthetic (seeded numpy default_rng(%d))' % w['seed'],
        'config': nuts_config(args, w, precision, world, eps),
        'min_ess_per_s': ess_s,
        'split_rhat_max_timed_draws': rhat,
        'lane_grads_profiled_pass': {
            'useful': prof['lf'], 'executed': prof['lf'],
            'lockstep_masked': w['chains'] * prof['leaves'] if prof['leaves'] else None,
            'leaf_iterations': prof['leaves'], 'transitions': args.steps},
        'step_size': eps,
        'mean_leapfrogs_per_chain_step': grad_evals / (args.steps * w['chains'] * world),
        'host_wall_s_timed_steps': wall,
        'e2e': {'value': e2e_value, 'unit': 'grad-evals/s', 'h2d_bytes_per_step': h2d,
                'd2h_bytes_per_step': d2h, 'steps': len(e2e_keys),
                'transitions': 'the timed transitions again, state in pinned host memory'},
        'roofline': roofline,
        'cpu_baseline': cpu,
        'other_precision': other,
        'gpu_launches': launches,
        'clocks': clk,
    }
    if prec_report is not None:
      line['precision_vs_fp64'] = prec_report
    print(json.dumps(line), flush=True)
  if dist is not None:
    dist.destroy_process_group()


def run_adapt(args, w):
  """Dual averaging over the whole adaptation window (num_adaptation_steps
  DA(NUTS) transitions, device loop) from the Laplace start at the initial
  step size; prints the step size the draws phase uses.  This is how the
  workloads' step_size_draws constants were obtained."""
  import torch
  import probability_gb300 as pg
  X, y, _ = make_data(w)
  init = laplace_start(X, y, w['chains'], w['seed'])
  precision = args.precision or w['precision']
  target = pg.LogisticRegression(engine_features(X, w), y, precision=precision)
  nuts = pg.mcmc.NoUTurnSampler(target, step_size=w['step0'], max_tree_depth=w['depth'])
  kernel = pg.mcmc.DualAveragingStepSizeAdaptation(
      nuts, num_adaptation_steps=w['num_adaptation_steps'],
      target_accept_prob=w['target_accept'])
  t0 = time.perf_counter()
  run = pg.mcmc.run_chain(kernel, 1, torch.from_numpy(init).cuda(),
                          num_burnin_steps=w['num_adaptation_steps'] - 1, seed=(w['seed'], 0))
  torch.cuda.synchronize()
  lar = run.trace['log_accept_ratio'].exp().clamp(max=1.0).mean().item()
  print(json.dumps({'adapt': args.workload, 'precision': precision,
                    'transitions': w['num_adaptation_steps'],
                    'step_size_draws': float(run.final_step_size.reshape(-1)[0].item()),
                    'last_mean_accept_prob': lar, 'seconds': time.perf_counter() - t0}),
        flush=True)


def make_batch_members(w):
  """The 256 posteriors (seeded numpy default_rng)."""
  rng = np.random.default_rng(w['seed'])
  spec = []
  for _ in range(w['mvn']):
    d = int(np.exp(rng.uniform(np.log(w['d_range'][0]), np.log(w['d_range'][1]))))
    A = rng.standard_normal((d, d + 2)) / np.sqrt(d)       # Wishart(d + 2, I / d)
    L = np.linalg.cholesky(A @ A.T)
    spec.append(('mvn', rng.normal(size=d), L, int(rng.integers(w['chains'][0],
                                                              w['chains'][1] + 1))))
  for _ in range(w['hier']):
    J = int(rng.integers(w['j_range'][0], w['j_range'][1] + 1))
    mu = rng.normal() * 5.0
    tau = abs(5.0 * np.tan(np.pi * (rng.uniform() - 0.5)))   # HalfCauchy(5)
    sigma = rng.uniform(5, 20, J)
    y = mu + tau * rng.normal(size=J) + sigma * rng.normal(size=J)
    spec.append(('hier', y, sigma, int(rng.integers(w['chains'][0], w['chains'][1] + 1))))
  return spec


def cpu_batch_gradient_rate(spec, max_seconds, sample=16, seed=0):
  """grad-evals/s of the oracle's log-density + gradient (NumPy, all host
  threads) over a seeded sample of the posteriors, each with its own chains:
  the NUTS leaf cost of those members on the CPU."""
  from oracle import targets as ot
  rng = np.random.default_rng(seed)
  pick = rng.choice(len(spec), size=min(sample, len(spec)), replace=False)
  members = []
  for i in pick:
    s = spec[i]
    t = ot.MultivariateNormalTriL(s[1], s[2]) if s[0] == 'mvn' else \
        ot.NonCentredHierarchicalNormal(s[1], s[2])
    d = t.dim if s[0] == 'mvn' else len(s[1]) + 2
    members.append((t, rng.normal(size=(s[3], d)) * 0.5))
  evals, passes = 0, 0
  t0 = time.perf_counter()
  while True:
    for t, x in members:
      t(x)
      evals += x.shape[0]
    passes += 1
    if time.perf_counter() - t0 > max_seconds:
      break
  dt = time.perf_counter() - t0
  return evals / dt, passes, dt, [int(i) for i in pick]


def run_batch(args, w):
  """256 uneven posteriors in one BatchedNoUTurnSampler."""
  import ctypes
  import torch
  import probability_gb300 as pg
  from probability_gb300 import _native
  from probability_gb300.batch import MemberDualAveraging, MemberMassMatrixAdaptation
  world, rank, local = dist_setup(args)
  if rank != 0:
    return
  dev = torch.device('cuda', local)
  torch.cuda.set_device(dev)
  t_setup = time.perf_counter()
  spec = make_batch_members(w)
  members = []
  for s in spec:
    if s[0] == 'mvn':
      members.append((pg.MultivariateNormalTriL(s[1], s[2]), s[3]))
    else:
      members.append((pg.NonCentredHierarchicalNormal(s[1], s[2]), s[3]))
  batch = pg.TargetBatch(members)
  rng = np.random.default_rng(w['seed'] + 1)
  q = batch.pack([torch.from_numpy((rng.normal(size=(c, t.event_dim)) * 0.5)
                                   .astype(np.float32)) for t, c in members]).to(dev)
  setup_s = time.perf_counter() - t_setup
  if args.kernel_only:   # the full-population gradient alone (profiling aid)
    for _ in range(args.warmup):
      batch.log_prob_and_grad(q)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(batch.stream)
    for _ in range(args.steps):
      batch.log_prob_and_grad(q)
    e1.record(batch.stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    flops = sum(2.0 * t.event_dim ** 2 * c if isinstance(t, pg.MultivariateNormalTriL)
                else 10.0 * t.groups * c for t, c in members)
    print(json.dumps({'kernel_only': True, 'workload': args.workload, 'ms_per_eval': ms,
                      'tflops': flops / ms / 1e9, 'chains': batch.chains,
                      'schedule': batch.schedule()}), flush=True)
    return
  da = MemberDualAveraging(batch, 0.1, args.warm_in, target_accept_prob=w['target_accept'])
  k = pg.BatchedNoUTurnSampler(batch, da.step_size, max_tree_depth=w['depth'])
  kr = k.bootstrap_results(q)
  t = 0
  # Warm-in: per-posterior dual averaging throughout; with preconditioning,
  # each posterior's diagonal metric is estimated over the middle third and
  # used from then on (a windowed adaptation, as windowed_sampling.py's).
  mm = MemberMassMatrixAdaptation(batch) if args.precondition else None
  w0, w1 = args.warm_in // 3, 2 * args.warm_in // 3
  for i in range(args.warm_in):
    q, kr = k.one_step(q, kr._replace(step_size=batch.per_chain(da.step_size)),
                       seed=pg._util.step_key((w['seed'], 0), t))
    da.update(kr.log_accept_ratio)
    t += 1
    if mm is not None and w0 <= i < w1:
      mm.update(q)
    if mm is not None and i == w1 - 1:
      k.set_inverse_mass(mm.inverse_mass())
  eps = batch.per_chain(da.step_size)
  kr = kr._replace(step_size=eps)
  for _ in range(args.warmup):
    q, kr = k.one_step(q, kr, seed=pg._util.step_key((w['seed'], 0), t))
    t += 1
  torch.cuda.synchronize()
  ms0, ev0, la0 = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
  read_profile = lambda ms_, ev_, la_: _native.lib().gbm_nuts_read_profile(
      k._handle, ctypes.byref(ms_), ctypes.byref(ev_), ctypes.byref(la_))
  flops_chain = torch.as_tensor(
      [2.0 * tt.event_dim ** 2 if isinstance(tt, pg.MultivariateNormalTriL)
       else 10.0 * tt.groups for tt, c in members for _ in range(c)], dtype=torch.float64,
      device=dev)
  l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
  C, E = batch.chains, batch.elements
  member_of_chain = torch.repeat_interleave(
      torch.arange(len(members), device=dev),
      torch.as_tensor(list(batch.member_chains), device=dev))

  def member_ess(states, prefix):
    """Sum over posteriors of the minimum (over coordinates) ESS of the
    member's draws states[:prefix[m]] (rows: transitions, ragged state);
    posteriors with fewer than 4 draws contribute 0."""
    total, counted = 0.0, 0
    for m in range(len(members)):
      P = int(prefix[m])
      if P < 4:
        continue
      e0_, n = int(batch.elem_begin[m]), batch.member_chains[m] * batch.member_dims[m]
      x = states[:P, e0_:e0_ + n].reshape(P, batch.member_chains[m], batch.member_dims[m])
      ess = pg.mcmc.effective_sample_size(x, filter_beyond_positive_pairs=True,
                                          cross_chain_dims=1)
      total += float(ess.min().item())
      counted += 1
    return total, counted

  clocks = ClockSampler(local)
  clocks.start()
  # ---- lock-step leg: BatchedNoUTurnSampler.one_step, every chain of every
  # posterior at the same tree depth and leaf ----
  lock_steps = max(1, min(args.steps, args.lock_steps))
  read_profile(ms0, ev0, la0)
  lf_total = torch.zeros((), dtype=torch.int64, device=dev)
  draws, step_ms, leaves = [], 0.0, 0
  torch.cuda.synchronize()
  for _ in range(lock_steps):
    l2_flush.zero_()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(batch.stream)
    q, kr = k.one_step(q, kr, seed=pg._util.step_key((w['seed'], 0), t))
    e1.record(batch.stream)
    t += 1
    leaves += k.last_leaf_iterations
    lf_total += kr.leapfrogs_taken.sum()
    draws.append(q)
    e1.synchronize()
    step_ms += e0.elapsed_time(e1)
  torch.cuda.synchronize()
  ms1, ev1, la1 = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
  read_profile(ms1, ev1, la1)
  lock_s = step_ms / 1000.0
  lock_ess = None
  if lock_steps >= 20:
    lock_ess, _ = member_ess(torch.stack(draws), [lock_steps] * len(members))
  del draws
  lock = {'value': int(lf_total.item()) / lock_s, 'unit': 'grad-evals/s', 'steps': lock_steps,
          'ms_per_step': step_ms / lock_steps, 'leaves_per_step': leaves / lock_steps,
          'sum_min_ess_per_s': (lock_ess / lock_s) if lock_ess is not None else None,
          'gpu_launches': int(la1.value),   # each read returns the count since the last
          'transitions': 'BatchedNoUTurnSampler.one_step: each step runs until the longest '
                         'trajectory of any chain ends (up to 1023 leaves at depth 10)'}
  # ---- free-running leg (timed, the line's value): BatchedNoUTurnSampler
  # .run_free with a fixed leaf-iteration budget; every chain starts its next
  # transition (keys step_key(seed, t0 + i)) as soon as its own trajectory
  # ends.  Only the leapfrogs of completed transitions count. ----
  budget = args.free_leaves
  kmax = args.free_transitions
  t0 = t
  ls0 = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
  read_profile(*ls0)
  l2_flush.zero_()
  torch.cuda.synchronize()
  f0 = torch.cuda.Event(enable_timing=True)
  f1 = torch.cuda.Event(enable_timing=True)
  f0.record(batch.stream)
  run = k.run_free(q, kr, kmax, (w['seed'], 0), first_step=t0, max_leaf_iterations=budget)
  f1.record(batch.stream)
  f1.synchronize()
  torch.cuda.synchronize()
  clk = clocks.stop()
  ls1 = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
  read_profile(*ls1)
  secs = f0.elapsed_time(f1) / 1000.0
  done = run.transitions_done.to(torch.int64)
  lf_tr = run.trace['leapfrogs_taken'].to(torch.int64)             # [kmax, C], 0 past done
  grad_evals = int(lf_tr.sum().item())
  flops = float((lf_tr.sum(0).to(torch.float64) * flops_chain).sum().item())
  prefix = torch.full((len(members),), 1 << 30, dtype=torch.int64, device=dev)
  prefix = prefix.scatter_reduce(0, member_of_chain, done, reduce='amin').cpu().tolist()
  ess_sum, ess_members = member_ess(run.all_states, prefix)
  done_cpu = done.cpu().numpy()
  free_stats = {'leaf_iteration_budget': budget, 'leaf_iterations': run.leaf_iterations,
                'max_transitions_per_chain': kmax,
                'transitions_per_chain': {'min': int(done_cpu.min()),
                                          'median': float(np.median(done_cpu)),
                                          'max': int(done_cpu.max())},
                'chains_at_max_transitions': int((done_cpu >= kmax).sum()),
                'member_common_prefix': {'min': int(min(prefix)), 'max': int(max(prefix))},
                'ess_members_with_4_or_more_draws': ess_members}
  del run
  # ---- end to end: run_free with the ragged state, log-densities and
  # gradients uploaded from pinned host memory, and each chain's last
  # completed state and transition count read back, every call ----
  e2e = None
  if args.steps > 0:
    e2e_budget = min(budget, 2 * 1023)
    e2e_k = 256   # above what any chain completes in the budget
    h_q = q.cpu().pin_memory()
    h_l = kr.target_log_prob.cpu().pin_memory()
    h_g = kr.grads_target_log_prob.cpu().pin_memory()
    h_out = torch.empty(E, dtype=torch.float32).pin_memory()
    h_done = torch.empty(C, dtype=torch.int32).pin_memory()
    elem_chain = torch.repeat_interleave(
        torch.arange(C, device=dev),
        torch.as_tensor(np.repeat(batch.member_dims, batch.member_chains), device=dev))
    elem_idx = torch.arange(E, device=dev)

    def e2e_call(seed_step):
      with torch.cuda.stream(batch.stream):
        dq = h_q.to(dev, non_blocking=True)
        kr2 = kr._replace(target_log_prob=h_l.to(dev, non_blocking=True),
                          grads_target_log_prob=h_g.to(dev, non_blocking=True))
      r = k.run_free(dq, kr2, e2e_k, (w['seed'], 0), first_step=seed_step,
                     max_leaf_iterations=e2e_budget)
      with torch.cuda.stream(batch.stream):
        d = r.transitions_done.to(torch.int64)
        last = (d[elem_chain] - 1).clamp_min(0)
        fin = torch.where(d[elem_chain] > 0, r.all_states[last, elem_idx], dq)
        h_out.copy_(fin, non_blocking=True)
        h_done.copy_(r.transitions_done, non_blocking=True)
        lf = int(r.trace['leapfrogs_taken'].to(torch.int64).sum().item())
      batch.stream.synchronize()
      return lf

    e2e_call(t0 + kmax)             # allocations for the trace outside the timed call
    torch.cuda.synchronize()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(batch.stream)
    lf_e = e2e_call(t0 + kmax + e2e_k)
    g1.record(batch.stream)
    g1.synchronize()
    e2e_s = g0.elapsed_time(g1) / 1000.0
    e2e = {'value': lf_e / e2e_s, 'unit': 'grad-evals/s',
           'h2d_bytes_per_step': E * 8 + C * 8, 'd2h_bytes_per_step': E * 4 + C * 4,
           'steps': 1, 'leaf_iteration_budget': e2e_budget,
           'transitions': 'BatchedNoUTurnSampler.run_free (%d leaf iterations) with the ragged '
                          'state, log-densities and gradients uploaded from pinned host memory '
                          'and each chain\'s last completed state and transition count read '
                          'back' % e2e_budget}
  achieved = flops / secs / 1e12
  fp32_peak = 2 * 128 * 152 * 2.07e9 / 1e12     # FMA lanes x 2 flop x SMs x max clock
  cpu = None
  if not args.no_cpu_baseline:
    budget_s = float(os.environ.get('GBM_CPU_BASELINE_SECONDS', '15'))
    rate, passes, dt, pick = cpu_batch_gradient_rate(spec, budget_s)
    cpu = {'value': rate, 'unit': 'grad-evals/s', 'cores': os.cpu_count(), 'kind': 'port',
           'sample': '%d passes of the log-prob+gradient of 16 of the 256 posteriors with all '
                     'their chains (%.1f s; the NUTS leaf cost, no tree bookkeeping); NumPy '
                     'float64 oracle targets, BLAS threads = all cores' % (passes, dt)}
  line = {
      'metric': METRIC_BATCH,
      'value': grad_evals / secs, 'unit': 'grad-evals/s', 'n_gpus': 1, 'steps': 1,
      'warmup': args.warmup, 'ms_per_step': secs * 1000.0, 'higher_is_better': True,
      'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32 (f64 energies)',
      'data': 'synthetic (seeded numpy default_rng(%d))' % w['seed'],
      'config': {'workload': args.workload, 'posteriors': len(members),
                 'mvn_dims': [int(tt.event_dim) for tt, _ in members[:w['mvn']]],
                 'chains_total': C, 'state_elements': E,
                 'max_tree_depth': w['depth'], 'warm_in_transitions': args.warm_in,
                 'step_size': 'one per posterior, dual averaging (target %.2f) in the warm-in'
                              % w['target_accept'],
                 'preconditioned': bool(args.precondition),
                 'chain_tile_schedule': batch.schedule(),
                 'timed': 'one free-running call (BatchedNoUTurnSampler.run_free) of %d leaf '
                          'iterations after %d lock-step warm-up and %d timed lock-step '
                          'transitions' % (budget, args.warmup, lock_steps),
                 'l2': 'flushed before each timed call (256 MB write outside the events)'},
      'sum_min_ess_per_s': ess_sum / secs,
      'free_running': free_stats,
      'lock_step': lock,
      'roofline': {'bound': 'fp32', 'achieved': achieved, 'peak': fp32_peak, 'unit': 'TFLOP/s',
                   'frac': achieved / fp32_peak, 'traffic': None,
                   'kernel': 'batch_phase_kernel (whole free-running call timed; flops of '
                             'completed transitions only)',
                   'peak_source': 'nominal FP32 FMA rate at the maximum SM clock'},
      'setup_s': setup_s, 'gpu_launches': int(ls1[2].value), 'clocks': clk,
      'cpu_baseline': cpu, 'e2e': e2e,
  }
  print(json.dumps(line), flush=True)

def serve_stream(pg, srv, jobs_spec, inputs, w, host):
  """Replay the stream through the job server.  host=False: each job's X, y
  and initial state are already on the device; host=True (end to end): they
  are uploaded from pinned host memory at submission and each job's draws
  are copied back to the host when it finishes, inside the timed window."""
  import torch
  from probability_gb300.serving import DONE
  handles = []
  t0 = time.perf_counter()
  for js, (X, y, q0) in zip(jobs_spec, inputs):
    delay = js['t'] - (time.perf_counter() - t0)
    if delay > 0:
      time.sleep(delay)
    if host:
      # The server's worker streams read these buffers: the upload completes
      # on the host's stream before the job is submitted.
      X, y, q0 = X.cuda(), y.cuda(), q0.cuda()
      torch.cuda.current_stream().synchronize()
    handles.append(srv.submit_logistic_regression(
        X, y, q0, js['draws'], precision='mixed', num_burnin_steps=js['adapt'],
        step_size=0.1, max_tree_depth=w['depth'], num_adaptation_steps=js['adapt'],
        target_accept_prob=0.8, seed=(w['seed'], js['seed']),
        trace=('state', 'leapfrogs_taken')))
  infos, d2h = [], 0
  for h in handles:
    infos.append(h.wait(timeout=7200.0))
    if host:
      st = h.states.cpu()
      d2h += st.numel() * 4
  wall = time.perf_counter() - t0
  assert all(i['status'] == DONE for i in infos)
  return handles, infos, wall, d2h


def run_serving(args, w):
  """Replay the head of a Poisson request stream through the job server and
  report latency percentiles, aggregate min-ESS/s and device throughput; then
  the same stream end to end from host memory."""
  import torch
  import probability_gb300 as pg
  from probability_gb300.serving import Server
  world, rank, local = dist_setup(args)
  if rank != 0:
    return
  dev = torch.device('cuda', local)
  torch.cuda.set_device(dev)
  rng = np.random.default_rng(w['seed'])
  R = int(os.environ.get('GBM_SERVE_REQUESTS', w['requests']))
  scale = float(os.environ.get('GBM_SERVE_LENGTH_SCALE', w['length_scale']))
  jobs_spec = []
  t_arr = 0.0
  for i in range(R):
    t_arr += rng.exponential(1.0 / w['rate'])
    n = int(np.exp(rng.uniform(np.log(w['n_range'][0]), np.log(w['n_range'][1]))))
    d = int(np.exp(rng.uniform(np.log(w['d_range'][0]), np.log(w['d_range'][1]))))
    c = int(rng.integers(w['chains'][0], w['chains'][1] + 1))
    draws = int(rng.integers(w['draws'][0], w['draws'][1] + 1))
    jobs_spec.append(dict(t=t_arr, n=n, d=d, c=c, draws=max(1, int(round(draws * scale))),
                          adapt=max(1, int(round(w['adapt'] * scale))), seed=i))
  # Inputs: seeded on the device (the device-resident pass does not time
  # their creation), with pinned host copies for the end-to-end pass.
  g = torch.Generator(device=dev)
  g.manual_seed(w['seed'])
  inputs = []
  for js in jobs_spec:
    X = torch.randn(js['n'], js['d'], device=dev, generator=g) * js['d'] ** -0.5
    X[:, 0] = 1.0
    beta = torch.randn(js['d'], device=dev, generator=g)
    y = (torch.rand(js['n'], device=dev, generator=g) < torch.sigmoid(X @ beta)).float()
    q0 = torch.randn(js['c'], js['d'], device=dev, generator=g) * 0.1
    inputs.append((X.to(torch.bfloat16), y, q0))
  torch.cuda.synchronize()
  srv = Server(workers=w['workers'], memory_budget_bytes=int(w['budget_gb'] * 2**30),
               device=local)
  clocks = ClockSampler(local)
  clocks.start()
  handles, infos, wall, _ = serve_stream(pg, srv, jobs_spec, inputs, w, host=False)
  clk = clocks.stop()
  lat = np.array([i['end_s'] - i['submit_s'] for i in infos])
  queue = np.array([i['start_s'] - i['submit_s'] for i in infos])
  busy = max(i['end_s'] for i in infos) - min(i['submit_s'] for i in infos)
  ess_sum, lf_sum, flops = 0.0, 0, 0.0
  per_job = []
  for js, h, inf in zip(jobs_spec, handles, infos):
    st = h.states                       # [draws, C, D]
    lf = int(h.leapfrogs_taken.sum().item())
    lf_sum += lf
    flops += 4.0 * js['n'] * js['d'] * lf
    ess_j = None
    if st.shape[0] >= 4:
      ess = pg.mcmc.effective_sample_size(st, filter_beyond_positive_pairs=True,
                                          cross_chain_dims=1)
      ess_j = float(ess.min().item())
      ess_sum += ess_j
    run_s = inf['end_s'] - inf['start_s']
    per_job.append([js['n'], js['d'], js['c'], js['draws'],
                    round(lf / (js['c'] * js['draws']), 1), round(run_s, 2),
                    round(4.0 * js['n'] * js['d'] * lf / run_s / 1e12, 1) if run_s > 0 else None,
                    round(ess_j, 1) if ess_j is not None else None])
  value = ess_sum / busy
  del handles
  e2e = None
  if args.serve_e2e:
    host_inputs = [(X.cpu().pin_memory(), y.cpu().pin_memory(), q0.cpu().pin_memory())
                   for X, y, q0 in inputs]
    h2, i2, wall2, d2h = serve_stream(pg, srv, jobs_spec, host_inputs, w, host=True)
    busy2 = max(i['end_s'] for i in i2) - min(i['submit_s'] for i in i2)
    ess2 = 0.0
    for h in h2:
      st = h.states
      if st.shape[0] >= 4:
        ess2 += float(pg.mcmc.effective_sample_size(
            st, filter_beyond_positive_pairs=True, cross_chain_dims=1).min().item())
    h2d = sum(X.numel() * 2 + y.numel() * 4 + q0.numel() * 4 for X, y, q0 in host_inputs)
    lat2 = np.array([i['end_s'] - i['submit_s'] for i in i2])
    e2e = {'value': ess2 / busy2, 'unit': 'ESS/s', 'h2d_bytes_per_step': h2d / R,
           'd2h_bytes_per_step': d2h / R,
           'latency_s': {'p50': float(np.percentile(lat2, 50)),
                         'p99': float(np.percentile(lat2, 99))},
           'note': 'the same stream with every job\'s X, y and initial state uploaded from '
                   'pinned host memory at submission and its draws copied back when it '
                   'finishes (a step is one request)'}
  srv.close()
  peaks, peak_src = read_peaks()
  achieved = flops / busy / 1e12
  roofline = {'bound': 'tensor', 'achieved': achieved, 'peak': peaks['bf16_tflops'],
              'unit': 'TFLOP/s', 'frac': achieved / peaks['bf16_tflops'], 'traffic': None,
              'kernel': 'all gradient kernels of the stream (aggregate over the makespan)',
              'peak_source': peak_src + ' (MEASURED_PEAKS.json bf16_tflops burst)',
              'note': 'algorithmic 4 N D flops per useful gradient evaluation summed over jobs, '
                      'divided by the makespan: a whole-stream utilisation (jobs are small and '
                      'latency-bound; sampler kernels and idle time are in the denominator)'}
  cpu = None
  if not args.no_cpu_baseline:
    # The oracle's batched log-prob + gradient (float32, all host threads) on
    # the first jobs' data and chains: the CPU cost of one NUTS leaf of those
    # jobs, turned into ESS/s with the GPU run's ESS per gradient evaluation.
    budget = float(os.environ.get('GBM_CPU_BASELINE_SECONDS', '20'))
    evals, secs = 0, 0.0
    for js, (X, y, q0) in list(zip(jobs_spec, inputs))[:4]:
      r, _, dt = cpu_gradient_rate(X.float().cpu().numpy(), y.cpu().numpy(),
                                   q0.cpu().numpy(), budget / 4)
      evals += r * dt
      secs += dt
    rate = evals / secs
    per_grad_ess = ess_sum / max(lf_sum, 1)
    cpu = {'value': rate * per_grad_ess, 'unit': 'ESS/s', 'cores': os.cpu_count(),
           'kind': 'port', 'grad_evals_per_s': rate,
           'sample': 'batched log-prob+gradient evaluations of the first 4 jobs (%.1f s), '
                     'float32 torch CPU ops, all host threads; ESS/s = that rate x the '
                     'stream\'s ESS per gradient evaluation on the GPU' % secs}
  line = {
      'metric': 'aggregate min-ESS/s over a served request stream (p50/p99 latency beside)',
      'value': value, 'unit': 'ESS/s', 'n_gpus': 1, 'steps': R, 'warmup': 0,
      'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'bf16+f32',
      'data': 'synthetic (seeded torch generator on the device)',
      'config': {'workload': args.workload, 'arrival_rate_per_s': w['rate'], 'requests': R,
                 'length_scale': scale, 'max_features': max(js['d'] for js in jobs_spec),
                 'jobs_above_512_features': int(sum(js['d'] > 512 for js in jobs_spec)),
                 'workers': w['workers'], 'memory_budget_gb': w['budget_gb'],
                 'max_tree_depth': w['depth'],
                 'note': 'the first %d requests of the Poisson stream at the stated lengths '
                         '(500-5000 draws after 300 adaptation steps) x %.2f' % (R, scale)},
      'latency_s': {'p50': float(np.percentile(lat, 50)), 'p99': float(np.percentile(lat, 99)),
                    'mean': float(lat.mean()), 'max': float(lat.max())},
      'queue_s': {'p50': float(np.percentile(queue, 50)), 'p99': float(np.percentile(queue, 99))},
      'makespan_s': busy, 'wall_s': wall, 'jobs_per_s': R / busy,
      'grad_evals_per_s': lf_sum / busy,
      'jobs': {'columns': ['rows', 'features', 'chains', 'draws', 'leapfrogs per chain and draw',
                           'run_s (adaptation + draws)', 'TFLOP/s of the draws over run_s',
                           'min_ess'], 'rows': per_job},
      'e2e': e2e, 'roofline': roofline, 'cpu_baseline': cpu,
      'clocks': clk,
  }
  print(json.dumps(line), flush=True)


def main():
  ap = argparse.ArgumentParser()
  ap.add_argument('--gpus', type=int, default=1)
  ap.add_argument('--steps', type=int, default=30)
  ap.add_argument('--warmup', type=int, default=5)
  ap.add_argument('--warm-in', type=int, default=100,
                  help='untimed dual-averaging transitions before warmup')
  ap.add_argument('--impl', default='engine', choices=['engine', 'reference'])
  ap.add_argument('--workload', default='nuts_logreg_1e5x100', choices=sorted(WORKLOADS))
  ap.add_argument('--precision', default=None, choices=[None, 'fp32', 'mixed'])
  ap.add_argument('--no-cpu-baseline', action='store_true')
  ap.add_argument('--other-precision', type=int, default=1,
                  help='also time the other precision (mixed beside FP32) on the same '
                       'transitions')
  ap.add_argument('--prewarm', type=int, default=6,
                  help='discarded transitions that capture leaf graphs before timing')
  ap.add_argument('--serve-e2e', type=int, default=1,
                  help='serving: replay the stream again end to end from host memory')
  ap.add_argument('--adapt', action='store_true',
                  help='run the adaptation window and print the draws-phase step size')
  ap.add_argument('--kernel-only', action='store_true',
                  help='time the batched log-prob+gradient alone (profiling aid)')
  ap.add_argument('--precondition', action='store_true',
                  help='nuts_batch_256: learn a diagonal metric per posterior in the warm-in')
  ap.add_argument('--lock-steps', type=int, default=20,
                  help='nuts_batch_256: timed lock-step transitions beside the free-running call')
  ap.add_argument('--free-leaves', type=int, default=10230,
                  help='nuts_batch_256: leaf-iteration budget of the timed free-running call')
  ap.add_argument('--free-transitions', type=int, default=512,
                  help='nuts_batch_256: transitions per chain at most in the free-running call')
  ap.add_argument('--kernel-rows', type=int, default=0,
                  help='with --kernel-only: rows of X (default: the workload\'s)')
  ap.add_argument('--kernel-shape', default='',
                  help='with --kernel-only: rows,features,chains (X drawn N(0, 1/features), '
                       'stored in the workload\'s data type)')
  args = ap.parse_args()
  w = WORKLOADS[args.workload]
  if args.adapt:
    run_adapt(args, w)
  elif args.impl == 'reference':
    run_reference(args, w)
  elif args.kernel_only and not args.workload.startswith('nuts_batch'):
    run_kernel_only(args, w)
  elif args.workload.startswith('hmc_'):
    run_hmc(args, w)
  elif args.workload.startswith('serve_'):
    run_serving(args, w)
  elif args.workload.startswith('nuts_batch'):
    run_batch(args, w)
  else:
    run_engine(args, w)


if __name__ == '__main__':
  main()
