"""Float64 exact solve of one MGPBD Newton system (TEST INFRASTRUCTURE).

Used only by tests/, tests/golden recipes and the oracle; never by the
product package.  It gives the solution of

    A dlam = b,   A = J W J^T + diag(alpha~)

that the reference's PCG (cons/mgpcg_gpu.py:261-329) approximates to its
stopping tolerance, so that positions of a substep can be checked against
the step with an exact linear solve rather than against another iterative
solver.  A is the reference's assembled matrix (cons/mgpbd_gpu.py:273-309):
J holds the constraint gradients per vertex slot (rows = constraints), W the
inverse vertex masses (zero for pinned vertices).

Method.  By the Woodbury identity, restricted to the free vertices F,

    A^-1 b = D^-1 (b - J_F y),   K y = J_F^T D^-1 b,
    K = W_F^-1 + J_F^T D^-1 J_F          (D = diag(alpha~)),

so the dual solve becomes a vertex-space solve with an SPD K (3 rows per
free vertex).  K is factorised (SuperLU) when it is small, otherwise it is
solved by CG preconditioned with its 3 x 3 vertex blocks.  Because D^-1
amplifies the primal error by up to 1/alpha~, the dual residual b - A dlam
is driven down by iterative refinement (each round solves for the
correction of the current residual) until it is below `tol` |b| in
float64.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla


def constraint_jacobian(t_i, grad, nv):
  """J (nc x 3 nv, CSR): row k holds grad[k, s] at the columns of vertex
  t_i[4k + s]; repeated slots of a constraint add up (their gradients are
  zero for the length constraints' repeated slots)."""
  q = np.asarray(t_i, np.int64).reshape(-1, 4)
  nc = len(q)
  g = np.asarray(grad, np.float64).reshape(nc, 4, 3)
  rows = np.repeat(np.arange(nc), 12)
  cols = (3 * q[:, :, None] + np.arange(3)[None, None, :]).reshape(-1)
  J = sp.csr_matrix((g.reshape(-1), (rows, cols)), shape=(nc, 3 * nv))
  J.sum_duplicates()
  return J


def block_jacobi(K):
  """Inverse 3 x 3 diagonal blocks of K (rows grouped by vertex) as a
  preconditioner."""
  n = K.shape[0] // 3
  C = K.tocoo()
  m = (C.row // 3) == (C.col // 3)
  B = np.zeros((n, 3, 3))
  np.add.at(B, (C.row[m] // 3, C.row[m] % 3, C.col[m] % 3), C.data[m])
  Bi = np.linalg.inv(B)
  return lambda r: np.einsum('nij,nj->ni', Bi, r.reshape(-1, 3)).reshape(-1)


def pcg(A, b, M, rtol=1e-13, maxiter=20000):
  """Preconditioned CG in float64; returns (x, iterations, relative residual)."""
  x = np.zeros_like(b)
  r = b.copy()
  nb = np.linalg.norm(b)
  if nb == 0.0:
    return x, 0, 0.0
  z = M(r)
  p = z.copy()
  rz = r @ z
  for k in range(maxiter):
    ap = A @ p
    alpha = rz / (p @ ap)
    x += alpha * p
    r -= alpha * ap
    if np.linalg.norm(r) <= rtol * nb:
      return x, k + 1, np.linalg.norm(r) / nb
    z = M(r)
    rz_new = r @ z
    p = z + (rz_new / rz) * p
    rz = rz_new
  return x, maxiter, np.linalg.norm(r) / nb


# ----------------------------------------------------------------------------
# the dual solve
# ----------------------------------------------------------------------------


class ExactDualSolve:
  """Solves A dlam = b for one Newton system (see module docstring).

  t_i: 4 vertex slots per constraint; grad: (nc, 4, 3) constraint
  gradients; invm: inverse masses (0 = pinned); alpha: alpha~ per
  constraint."""

  DIRECT_MAX = 60000  # K rows up to which SuperLU factorises K

  def __init__(self, t_i, grad, invm, alpha, direct_max=None):
    invm = np.asarray(invm, np.float64)
    nv = len(invm)
    self.alpha = np.asarray(alpha, np.float64)
    self.J = constraint_jacobian(t_i, grad, nv)
    free_v = invm > 0
    free = np.repeat(free_v, 3)
    self.w = np.repeat(invm, 3)
    self.JF = self.J[:, free].tocsr()
    self.JFt = self.JF.T.tocsr()
    dinv = 1.0 / self.alpha
    self.dinv = dinv
    K = (sp.diags(1.0 / self.w[free]) + self.JFt @ sp.diags(dinv) @ self.JF).tocsc()
    self.K = K.tocsr()
    self.iters = []
    lim = self.DIRECT_MAX if direct_max is None else direct_max
    if K.shape[0] <= lim:
      lu = sla.splu(K, permc_spec='MMD_AT_PLUS_A')
      self._primal = lambda r: (lu.solve(r), 0)
    else:
      M = block_jacobi(self.K)

      def primal(r):
        y, it, _ = pcg(self.K, r, M, rtol=1e-14, maxiter=200000)
        return y, it

      self._primal = primal

  def apply_A(self, v):
    return self.alpha * v + self.J @ (self.w * (self.J.T @ v))

  def solve(self, b, tol=1e-11, max_rounds=8):
    """dlam with |b - A dlam| <= tol |b| (float64), by Woodbury solves of the
    residual with iterative refinement; returns (dlam, relative residual)."""
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    dlam = np.zeros_like(b)
    if nb == 0.0:
      return dlam, 0.0
    r = b.copy()
    rel = 1.0
    for _ in range(max_rounds):
      y, it = self._primal(self.JFt @ (self.dinv * r))
      self.iters.append(it)
      dlam += self.dinv * (r - self.JF @ y)
      r = b - self.apply_A(dlam)
      rel = np.linalg.norm(r) / nb
      if rel <= tol:
        break
    return dlam, rel


# ----------------------------------------------------------------------------
# the FAST step's linear solve, restated in float64
# ----------------------------------------------------------------------------


def chebyshev_pcg(apply_A, b, degree=8, lo=1e-3, scale=None, rel_tol=1e-6, tol_abs=0.0,
                  maxiter=6000, lmax=None, x0=None):
  """CG preconditioned by a degree-`degree` Chebyshev polynomial in S A
  (S = diag(scale), or the identity) on [lo * 1.02 lmax, 1.02 lmax], lmax
  the largest eigenvalue of S A (Lanczos to 1e-10 unless given), from
  x = 0 (or x0: the library's warm start), until |r| < max(tol_abs,
  rel_tol |b|): the linear solve of the library's FAST mode in float64.
  Returns (x, iterations)."""
  b = np.asarray(b, np.float64)
  n = len(b)
  sc = np.ones(n) if scale is None else np.asarray(scale, np.float64)
  if lmax is None:
    op = sla.LinearOperator((n, n), matvec=lambda v: np.sqrt(sc) * apply_A(np.sqrt(sc) * v),
                            dtype=np.float64)
    lmax = float(sla.eigsh(op, k=1, which='LA', tol=1e-10, return_eigenvectors=False)[0])
  hi = 1.02 * lmax
  a_ = lo * hi
  theta, delta = 0.5 * (hi + a_), 0.5 * (hi - a_)
  sigma = theta / delta

  def precond(r):
    x = np.zeros_like(r)
    rr = r.copy()
    d = sc * rr / theta
    rho = 1.0 / sigma
    for _ in range(degree):
      x += d
      rr -= apply_A(d)
      rho_n = 1.0 / (2.0 * sigma - rho)
      d = rho_n * rho * d + 2.0 * rho_n / delta * (sc * rr)
      rho = rho_n
    return x

  x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
  r = b.copy() if x0 is None else b - apply_A(x)
  tol = max(tol_abs, rel_tol * np.linalg.norm(b))
  if np.linalg.norm(r) < tol:
    return x, 0
  z = precond(r)
  p = z.copy()
  rz = r @ z
  for k in range(maxiter):
    ap = apply_A(p)
    alpha = rz / (p @ ap)
    x += alpha * p
    r -= alpha * ap
    if np.linalg.norm(r) < tol:
      return x, k + 1
    z = precond(r)
    rz_new = r @ z
    p = z + (rz_new / rz) * p
    rz = rz_new
  return x, maxiter


def chebyshev_pcg_bodies(apply_A, b, bodies, degree=8, lo=1e-3, rel_tol=1e-6, tol_abs=0.0,
                         maxiter=6000, lmax=None):
  """One Chebyshev-preconditioned CG per body on a block-diagonal A, in
  lockstep with one shared polynomial (lmax of the whole A), as the
  library's per-body kernel runs them: each body's dot products, alpha,
  beta and stopping test (|r_b| < max(tol_abs, rel_tol |b_b|)) are its own,
  and a body that stops keeps its x and r.  bodies: one index array per
  body (together a partition).  Returns (x, per-body iterations)."""
  b = np.asarray(b, np.float64)
  n = len(b)
  if lmax is None:
    op = sla.LinearOperator((n, n), matvec=apply_A, dtype=np.float64)
    lmax = float(sla.eigsh(op, k=1, which='LA', tol=1e-10, return_eigenvectors=False)[0])
  hi = 1.02 * lmax
  a_ = lo * hi
  theta, delta = 0.5 * (hi + a_), 0.5 * (hi - a_)
  sigma = theta / delta

  def precond(r):
    x = np.zeros_like(r)
    rr = r.copy()
    d = rr / theta
    rho = 1.0 / sigma
    for _ in range(degree):
      x += d
      rr -= apply_A(d)
      rho_n = 1.0 / (2.0 * sigma - rho)
      d = rho_n * rho * d + 2.0 * rho_n / delta * rr
      rho = rho_n
    return x

  nb = len(bodies)
  x = np.zeros(n)
  r = b.copy()
  tol = [max(tol_abs, rel_tol * np.linalg.norm(b[ix])) for ix in bodies]
  done = [bool(np.linalg.norm(r[ix]) < tol[k]) for k, ix in enumerate(bodies)]
  its = [0] * nb
  z = precond(r)
  p = z.copy()
  rz = [r[ix] @ z[ix] for ix in bodies]
  for _ in range(maxiter):
    if all(done):
      break
    ap = apply_A(p)
    for k, ix in enumerate(bodies):
      if done[k]:
        continue
      alpha = rz[k] / (p[ix] @ ap[ix])
      x[ix] += alpha * p[ix]
      r[ix] -= alpha * ap[ix]
      its[k] += 1
      if np.linalg.norm(r[ix]) < tol[k]:
        done[k] = True
    z = precond(r)
    for k, ix in enumerate(bodies):
      if done[k]:
        continue
      rz_new = r[ix] @ z[ix]
      p[ix] = z[ix] + (rz_new / rz[k]) * p[ix]
      rz[k] = rz_new
  return x, its
