"""Window schedule of WindowedAdaptation (experimental/mcmc/windowed_sampling.py:
322-347): for 500 adaptation steps a first fast window of 75 steps, slow
windows of 25, 50, 100 and 200 and a last fast window of 50 -- the schedule
the reference's docstring states."""
from probability_gb300.experimental.mcmc import _get_window_sizes


def test_window_sizes_match_reference_schedule():
  first, slow, last = _get_window_sizes(500)
  assert (first, slow, last) == (75, 25, 50)
  assert first + slow * (1 + 2 + 4 + 8) + last == 500
  for n in (100, 237, 1000, 2001):
    f, s, l = _get_window_sizes(n)
    assert f == 3 * s and f + 15 * s + l == n and l >= 0
