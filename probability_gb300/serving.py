"""Serving many posteriors at once on one GPU (C ABI: gbm_server_*).

A ``Server`` admits posterior-sampling jobs first-in first-out under a
device-memory budget and runs admitted jobs concurrently on its workers'
private streams; every job is a DualAveragingStepSizeAdaptation(NoUTurnSampler)
sample_chain run whose chain and adaptation state stay on the device until it
finishes.  Kernels are deterministic, so a job's draws are the same whether it
runs alone or beside other jobs.
"""
import ctypes

import torch

from probability_gb300 import _native, _util

QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3
_FAMILY = dict(logistic_regression=0, mvn=1, hierarchical_normal=2)

P = ctypes.c_void_p


class JobSpec(ctypes.Structure):
  _fields_ = [
      ('family', ctypes.c_int32), ('x', P), ('x_dtype', ctypes.c_int32),
      ('precision', ctypes.c_int32), ('rows', ctypes.c_int64), ('features', ctypes.c_int64),
      ('y', P), ('prior_scale', ctypes.c_float), ('loc', P), ('scale_tril_inv', P),
      ('log_normalizer', ctypes.c_double), ('group_y', P), ('group_sigma', P),
      ('groups', ctypes.c_int64), ('mu_scale', ctypes.c_float), ('tau_scale', ctypes.c_float),
      ('dim', ctypes.c_int64), ('chains', ctypes.c_int64), ('init_state', P),
      ('step_size', ctypes.c_float), ('max_tree_depth', ctypes.c_int32),
      ('num_adaptation_steps', ctypes.c_int32), ('target_accept_prob', ctypes.c_double),
      ('num_results', ctypes.c_int64), ('num_burnin_steps', ctypes.c_int64),
      ('seed', ctypes.c_uint32 * 2), ('trace_state', P), ('trace_log_accept_ratio', P),
      ('trace_leapfrogs_taken', P), ('final_state', P), ('final_step_size', P),
      ('moments_mean', P), ('moments_m2', P),
  ]


class JobInfo(ctypes.Structure):
  _fields_ = [('status', ctypes.c_int32), ('error_code', ctypes.c_int32),
              ('submit_s', ctypes.c_double), ('start_s', ctypes.c_double),
              ('end_s', ctypes.c_double), ('device_bytes', ctypes.c_int64)]


_SIGS = {
    'gbm_server_create': ([ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(P)],
                          ctypes.c_int),
    'gbm_server_destroy': ([P], ctypes.c_int),
    'gbm_server_submit': ([P, ctypes.POINTER(JobSpec), ctypes.POINTER(ctypes.c_int64)],
                          ctypes.c_int),
    'gbm_server_query': ([P, ctypes.c_int64, ctypes.POINTER(JobInfo)], ctypes.c_int),
    'gbm_server_wait': ([P, ctypes.c_int64, ctypes.c_double, ctypes.POINTER(JobInfo)],
                        ctypes.c_int),
    'gbm_server_release': ([P, ctypes.c_int64], ctypes.c_int),
    'gbm_server_now': ([P], ctypes.c_double),
}


def _lib():
  L = _native.lib()
  if not getattr(L, '_server_sigs', False):
    for name, (args, res) in _SIGS.items():
      fn = getattr(L, name)
      fn.argtypes = args
      fn.restype = res
    L._server_sigs = True
  return L


class Job:
  """Handle to a submitted job; outputs are device tensors filled on DONE."""

  def __init__(self, server, job_id, keep, outputs):
    self.server = server
    self.id = job_id
    self._keep = keep            # inputs must outlive the job
    self.outputs = outputs

  def info(self):
    inf = JobInfo()
    _native.check(_lib().gbm_server_query(self.server._h, self.id, ctypes.byref(inf)),
                  'gbm_server_query')
    return _info_dict(inf)

  def wait(self, timeout=3600.0):
    inf = JobInfo()
    st = _lib().gbm_server_wait(self.server._h, self.id, float(timeout), ctypes.byref(inf))
    _native.check(st, 'gbm_server_wait')
    d = _info_dict(inf)
    if d['status'] == FAILED:
      _native.check(d['error_code'] or _native.GBM_ECUDA, 'job %d' % self.id)
    return d

  def __getattr__(self, name):
    outs = self.__dict__.get('outputs', {})
    if name in outs:
      return outs[name]
    raise AttributeError(name)


def _info_dict(inf):
  return dict(status=inf.status, error_code=inf.error_code, submit_s=inf.submit_s,
              start_s=inf.start_s, end_s=inf.end_s, device_bytes=inf.device_bytes,
              latency_s=inf.end_s - inf.submit_s if inf.status in (DONE, FAILED) else None,
              queue_s=inf.start_s - inf.submit_s if inf.status != QUEUED else None)


class Server:
  """gbm_server: ``workers`` concurrent jobs, FIFO admission under
  ``memory_budget_bytes`` of (estimated) device memory."""

  def __init__(self, workers=8, memory_budget_bytes=150 * 2**30, device=None):
    dev = _util.device() if device is None else torch.device('cuda', device)
    h = P()
    _native.check(_lib().gbm_server_create(dev.index, int(workers), int(memory_budget_bytes),
                                           ctypes.byref(h)), 'gbm_server_create')
    self._h = h
    self.device = dev

  def now(self):
    return _lib().gbm_server_now(self._h)

  def close(self):
    if self._h is not None:
      _lib().gbm_server_destroy(self._h)
      self._h = None

  def __del__(self):
    try:
      self.close()
    except Exception:
      pass

  def _submit(self, spec, keep, init_state, num_results, num_burnin_steps, step_size,
              max_tree_depth, num_adaptation_steps, target_accept_prob, seed, trace):
    q = _util.as_tensor(init_state, torch.float32, self.device)
    C, D = q.shape
    R = int(num_results)
    dev = self.device
    outs = dict(final_state=torch.empty((C, D), dtype=torch.float32, device=dev),
                final_step_size=torch.empty(1, dtype=torch.float32, device=dev))
    if 'state' in trace:
      outs['states'] = torch.empty((R, C, D), dtype=torch.float32, device=dev)
    if 'log_accept_ratio' in trace:
      outs['log_accept_ratio'] = torch.empty((R, C), dtype=torch.float64, device=dev)
    if 'leapfrogs_taken' in trace:
      outs['leapfrogs_taken'] = torch.empty((R, C), dtype=torch.int32, device=dev)
    if 'moments' in trace:   # streaming per-chain mean / squared deviations of the draws
      outs['moments_mean'] = torch.empty((C, D), dtype=torch.float64, device=dev)
      outs['moments_m2'] = torch.empty((C, D), dtype=torch.float64, device=dev)
    seed = _util.sanitize_seed(seed)
    spec.dim, spec.chains, spec.init_state = D, C, _native.ptr(q)
    spec.step_size = float(step_size)
    spec.max_tree_depth = int(max_tree_depth)
    spec.num_adaptation_steps = int(num_adaptation_steps)
    spec.target_accept_prob = float(target_accept_prob)
    spec.num_results, spec.num_burnin_steps = R, int(num_burnin_steps)
    spec.seed[0], spec.seed[1] = seed
    spec.trace_state = _native.ptr(outs.get('states'))
    spec.trace_log_accept_ratio = _native.ptr(outs.get('log_accept_ratio'))
    spec.trace_leapfrogs_taken = _native.ptr(outs.get('leapfrogs_taken'))
    spec.moments_mean = _native.ptr(outs.get('moments_mean'))
    spec.moments_m2 = _native.ptr(outs.get('moments_m2'))
    spec.final_state = _native.ptr(outs['final_state'])
    spec.final_step_size = _native.ptr(outs['final_step_size'])
    # Inputs were written on this thread's torch stream; the workers use their
    # own streams, so make the inputs visible before handing them over.
    torch.cuda.current_stream(dev).synchronize()
    jid = ctypes.c_int64()
    _native.check(_lib().gbm_server_submit(self._h, ctypes.byref(spec), ctypes.byref(jid)),
                  'gbm_server_submit')
    return Job(self, jid.value, keep + [q], outs)

  def submit_logistic_regression(self, features, labels, init_state, num_results,
                                 prior_scale=1.0, precision='mixed', **kw):
    X = _util.as_tensor(features, None, self.device)
    if precision == 'fp32' or X.dtype not in (torch.float32, torch.bfloat16):
      X = X.to(torch.float32)
    y = _util.as_tensor(labels, torch.float32, self.device).reshape(-1)
    s = JobSpec()
    s.family = _FAMILY['logistic_regression']
    s.x = _native.ptr(X)
    s.x_dtype = _native.DTYPE_BF16 if X.dtype == torch.bfloat16 else _native.DTYPE_F32
    s.precision = _native.PRECISION_MIXED if precision == 'mixed' else _native.PRECISION_F32
    s.rows, s.features = X.shape
    s.y = _native.ptr(y)
    s.prior_scale = float(prior_scale)
    return self._submit(s, [X, y], init_state, num_results, **_defaults(kw))

  def submit_mvn(self, loc, scale_tril, init_state, num_results, **kw):
    import numpy as np
    import scipy.linalg
    L = np.asarray(_util.as_tensor(scale_tril, torch.float64).cpu().numpy())
    d = L.shape[0]
    Linv = scipy.linalg.solve_triangular(np.tril(L), np.eye(d), lower=True)
    s = JobSpec()
    s.family = _FAMILY['mvn']
    loc_t = _util.as_tensor(loc, torch.float32, self.device).reshape(-1)
    li = _util.as_tensor(np.tril(Linv), torch.float32, self.device)
    s.loc, s.scale_tril_inv = _native.ptr(loc_t), _native.ptr(li)
    s.log_normalizer = float(-np.sum(np.log(np.abs(np.diag(L)))) - 0.5 * d * np.log(2 * np.pi))
    return self._submit(s, [loc_t, li], init_state, num_results, **_defaults(kw))

  def submit_hierarchical_normal(self, y, sigma, init_state, num_results, mu_scale=5.0,
                                 tau_scale=5.0, **kw):
    s = JobSpec()
    s.family = _FAMILY['hierarchical_normal']
    y_t = _util.as_tensor(y, torch.float32, self.device).reshape(-1)
    s_t = _util.as_tensor(sigma, torch.float32, self.device).reshape(-1)
    s.group_y, s.group_sigma, s.groups = _native.ptr(y_t), _native.ptr(s_t), y_t.shape[0]
    s.mu_scale, s.tau_scale = float(mu_scale), float(tau_scale)
    return self._submit(s, [y_t, s_t], init_state, num_results, **_defaults(kw))


def _defaults(kw):
  out = dict(num_burnin_steps=0, step_size=0.1, max_tree_depth=10, num_adaptation_steps=0,
             target_accept_prob=0.8, seed=(0, 0), trace=('state', 'log_accept_ratio',
                                                         'leapfrogs_taken'))
  unknown = set(kw) - set(out)
  if unknown:
    raise TypeError('unknown job arguments: %s' % sorted(unknown))
  out.update(kw)
  return out
