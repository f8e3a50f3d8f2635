"""The device's largest-eigenvalue search for the Chebyshev interval
(`lanczos_lmax` in csrc/jform.cu: Sturm-sequence multisection of the
Lanczos tridiagonal, one warp, 32 probes per round), restated step for step
in numpy and checked on the CPU against dense eigenvalues.

Each round the 32 probes split the current interval into 33 parts; lane l
probes lo + (l + 1) (hi - lo) / 33 (lane 31: hi - (hi - lo) / 33); the
first probe with every eigenvalue below it is the new upper end, the probe
before it (or the old lower end) the new lower end; a round with no such
probe keeps the upper end and moves the lower end to the last probe.  The
search stops when the width is below 1e-12 of max(1, |hi|), and returns the
upper end.  The GPU path is exercised by every Chebyshev solve of the
`-m gpu` suite; this test pins the interval logic itself, including
tridiagonals with zero off-diagonals, negative and repeated eigenvalues.
"""

import numpy as np
import pytest


def sturm_below(a, b, x):
  """Eigenvalues of the tridiagonal (a, b) below x (the kernel's recurrence,
  with its zero pivot replaced by -1e-300)."""
  c = 0
  d = 1.0
  for i in range(len(a)):
    q = (b[i - 1] * b[i - 1]) / d if i > 0 else 0.0
    d = (a[i] - x) - q
    if d == 0.0:
      d = -1e-300
    if d < 0.0:
      c += 1
  return c


def lmax_multisection(a, b):
  k = len(a)
  lo, hi = 1e300, -1e300
  for i in range(k):
    r = (abs(b[i - 1]) if i > 0 else 0.0) + (abs(b[i]) if i + 1 < k else 0.0)
    lo = min(lo, a[i] - r)
    hi = max(hi, a[i] + r)
  for _ in range(60):
    if not hi - lo > 1e-12 * max(1.0, abs(hi)):
      break
    step = (hi - lo) / 33.0
    xs = [lo + step * (l + 1) for l in range(31)] + [hi - step]
    allbelow = [sturm_below(a, b, x) >= k for x in xs]
    f = allbelow.index(True) if any(allbelow) else 32
    nlo = lo if f == 0 else xs[f - 1]
    nhi = hi if f == 32 else xs[f]
    lo, hi = nlo, nhi
  return hi


def tridiag_eigmax(a, b):
  T = np.diag(a) + np.diag(b[:len(a) - 1], 1) + np.diag(b[:len(a) - 1], -1)
  return float(np.linalg.eigvalsh(T).max())


@pytest.mark.parametrize('seed', range(6))
def test_multisection_finds_the_largest_eigenvalue(seed):
  rng = np.random.default_rng(seed)
  k = int(rng.integers(2, 33))
  a = rng.uniform(-2.0, 10.0, k) * 10.0 ** rng.uniform(-3, 3)
  b = rng.uniform(-1.0, 1.0, k) * 10.0 ** rng.uniform(-3, 1)
  got = lmax_multisection(a, b)
  want = tridiag_eigmax(a, b)
  assert got >= want - 1e-12 * max(1.0, abs(want))  # an upper end
  assert abs(got - want) <= 2e-12 * max(1.0, abs(want)), (got, want)


def test_multisection_edge_cases():
  # diagonal (no coupling), repeated, one row, all negative
  for a, b in [(np.array([1.0, 5.0, 3.0]), np.zeros(3)),
               (np.full(8, 2.0), np.zeros(8)),
               (np.array([4.5]), np.zeros(1)),
               (np.array([-3.0, -1.0, -2.0]), np.array([0.5, 0.25, 0.0]))]:
    got = lmax_multisection(a, b)
    want = tridiag_eigmax(a, b)
    assert abs(got - want) <= 2e-12 * max(1.0, abs(want)), (a, b, got, want)


def test_multisection_on_a_lanczos_tridiagonal():
  """24 Lanczos steps on an SPD matrix with a spread spectrum (as the
  library runs on D^-1/2 A D^-1/2): the tridiagonal's largest eigenvalue,
  found by the multisection, is the matrix's to 1e-6."""
  rng = np.random.default_rng(3)
  n = 400
  ev = np.concatenate([np.linspace(1e-3, 1.0, n - 1), [3.7]])
  Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
  A = (Q * ev) @ Q.T
  q = rng.standard_normal(n)
  q /= np.linalg.norm(q)
  qprev = np.zeros(n)
  a, b = [], []
  beta = 0.0
  for _ in range(24):
    w = A @ q - beta * qprev
    alpha = q @ w
    w -= alpha * q
    beta = np.linalg.norm(w)
    a.append(alpha)
    b.append(beta)
    qprev, q = q, w / beta
  got = lmax_multisection(np.array(a), np.array(b))
  assert abs(got - 3.7) <= 1e-6 * 3.7
