"""Elementwise bijectors for TransformedTransitionKernel.

The subset of tfp.bijectors that maps an unconstrained real state onto a
constrained support elementwise (bijectors/exp.py, softplus.py, sigmoid.py,
identity.py).  ``forward``/``inverse`` are torch functions used to move
states between the two spaces; the sampler's hot path applies the forward
map and its log-Jacobian inside the engine (gbm_target_transformed).
"""
import torch

IDENTITY, EXP, SOFTPLUS, SIGMOID = 0, 1, 2, 3


class Bijector:
  code = IDENTITY
  name = 'identity'

  def forward(self, x):
    return x

  def inverse(self, y):
    return y

  def __repr__(self):
    return 'tfb.%s()' % type(self).__name__


class Identity(Bijector):
  pass


class Exp(Bijector):
  """y = exp(x) (bijectors/exp.py)."""
  code, name = EXP, 'exp'

  def forward(self, x):
    return torch.exp(x)

  def inverse(self, y):
    return torch.log(y)


class Softplus(Bijector):
  """y = log(1 + exp(x)) (bijectors/softplus.py, hinge_softness = 1)."""
  code, name = SOFTPLUS, 'softplus'

  def forward(self, x):
    return torch.nn.functional.softplus(x)

  def inverse(self, y):
    # log(exp(y) - 1) = y + log(1 - exp(-y)), stable for large y
    return y + torch.log(-torch.expm1(-y))


class Sigmoid(Bijector):
  """y = 1 / (1 + exp(-x)) (bijectors/sigmoid.py, on (0, 1))."""
  code, name = SIGMOID, 'sigmoid'

  def forward(self, x):
    return torch.sigmoid(x)

  def inverse(self, y):
    return torch.log(y) - torch.log1p(-y)
