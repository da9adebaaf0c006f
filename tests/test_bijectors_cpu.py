"""The Python bijectors (state transport for TransformedTransitionKernel)
against the oracle's forward maps (bijectors/exp.py, softplus.py, sigmoid.py)
and their own inverses, on CPU tensors."""
import numpy as np
import pytest
import torch

import probability_gb300 as pg
from oracle import targets

_B = [pg.bijectors.Identity(), pg.bijectors.Exp(), pg.bijectors.Softplus(),
      pg.bijectors.Sigmoid()]


@pytest.mark.parametrize('b', _B, ids=lambda b: b.name)
def test_forward_matches_oracle_and_inverts(b):
  x = np.linspace(-12.0, 12.0, 241)
  y = b.forward(torch.from_numpy(x)).numpy()
  codes = np.full(x.shape, b.code)
  want = targets.TransformedTarget(None, codes).forward(x[None, :])[0]
  # atol: the oracle's sigmoid, 0.5 (1 + tanh(x / 2)), carries ~4e-17 absolute
  # error in the far negative tail.
  np.testing.assert_allclose(y, want, rtol=1e-13, atol=1e-15)
  keep = np.abs(x) <= (12.0 if b.code != pg.bijectors.SIGMOID else 10.0)   # sigmoid saturates
  back = b.inverse(torch.from_numpy(y)).numpy()
  np.testing.assert_allclose(back[keep], x[keep], rtol=1e-9, atol=1e-9)


def test_codes_are_the_engine_codes():
  # The codes index the engine's bijector switch (GBM_BIJECTOR_* in gb300_mcmc.h).
  assert [b.code for b in _B] == [0, 1, 2, 3]
