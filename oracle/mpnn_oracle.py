"""CPU restatement of the learned coarse correction, for checking only.

TEST INFRASTRUCTURE: the oracle the CUDA network kernels (`csrc/mpnn.cu`)
are compared against.  Imported by tests/ only; the product package never
imports it.

The reference has no learned component: its V-cycle's coarse correction is
`min(50, n)` weighted-Jacobi sweeps on the coarsest level
(cons/mgpcg_gpu.py:216-224) of the two-level tet-aggregation hierarchy
(cons/tet_aggregation.py:145-211).  The learned correction replaces it by a
linear operator whose per-aggregate weights a message-passing network
computes from the graph of the level-1 matrix A_c (once per matrix):

  e_c = w * (r_c / diag(A_c))

Network (n aggregates, F = 64 hidden features), on a scalar node field r:

  s_i   = sqrt(1 / A_ii)          (0 where A_ii <= 0)
  Ah    = S A S                   (symmetric, unit diagonal)
  sigma = sqrt(sum_i (s_i r_i)^2 / n)          (output 0 when sigma == 0)
  u     = S r / sigma,   a1 = Ah u
  H1    = relu(u w1s^T + a1 w1n^T + 1 b1^T)                   (n, F)
  G1    = Ah H1,  H2 = relu([H1, G1] W2 + 1 b2^T)              W2: (2F, F)
  G2    = Ah H2,  H3 = relu([H2, G2] W3 + 1 b3^T)
  y     = H3 wo + bo,            e = sigma S y

The weights come from the network's y on the field r_i = sqrt(A_ii) (so
u = 1 and a1 = the row sums of Ah), squashed into (0, c_i):

  w_i = c_i * sigmoid(y_i),   c_i = 1.9 / R_i,   R_i = sum_j |Ah_ij|.

Below 2 / R_i the correction cannot over-correct any mode (Gershgorin:
2 W^-1 - Ah stays diagonally dominant, so B = W D^-1 satisfies B < 2 A^-1
and the V-cycle stays positive definite); the l1-Jacobi weight is 1 / R_i.

Training minimises the scaled coarse energy of the correction over a batch
of restricted residuals r_s: with u_s = S r_s / sigma_s and v_s = w * u_s
(the scaled correction, w the projected weights),

  L = mean_s (1/2 v_s^T Ah v_s - v_s^T u_s) / n,

and E(e) - E(A_c^-1 r) is half the squared energy-norm error of e, so the
loss ranks corrections without exact solves.  `forward`/`loss_and_grad`
(`mode='field'`) keep the network's plain use on a residual field, e = net(r)
with L = mean_s (1/2 y^T Ah y - y^T u_s) / n, which checks the same kernels.

`device=True` reproduces the storage precision of the CUDA kernels: W2, W3
and the activations H1, G1, H2, G2 are rounded to bfloat16 (round to
nearest even), everything else is float32/float64 arithmetic.  With
`device=False` the whole network is float64 (for finite-difference checks).

Parameter vector layout (float32, 16,769 values), shared with the library:
  w1s[64] w1n[64] b1[64] | W2[128][64] b2[64] | W3[128][64] b3[64] | wo[64] bo
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

F = 64
OFF_W1S, OFF_W1N, OFF_B1 = 0, 64, 128
OFF_W2 = 192
OFF_B2 = OFF_W2 + 2 * F * F
OFF_W3 = OFF_B2 + F
OFF_B3 = OFF_W3 + 2 * F * F
OFF_WO = OFF_B3 + F
OFF_BO = OFF_WO + F
N_PARAMS = OFF_BO + 1


def bf16(x):
  """Round float32 values to bfloat16 (nearest even), returned as float32."""
  a = np.ascontiguousarray(np.asarray(x, np.float32))
  b = a.view(np.uint32).astype(np.uint64)
  b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
  return b.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p):
  p = np.asarray(p, np.float64)
  return {
      'w1s': p[OFF_W1S:OFF_W1S + F], 'w1n': p[OFF_W1N:OFF_W1N + F], 'b1': p[OFF_B1:OFF_B1 + F],
      'W2': p[OFF_W2:OFF_B2].reshape(2 * F, F), 'b2': p[OFF_B2:OFF_B2 + F],
      'W3': p[OFF_W3:OFF_B3].reshape(2 * F, F), 'b3': p[OFF_B3:OFF_B3 + F],
      'wo': p[OFF_WO:OFF_WO + F], 'bo': p[OFF_BO]}


def pack(d):
  p = np.zeros(N_PARAMS, np.float64)
  p[OFF_W1S:OFF_W1S + F] = d['w1s']
  p[OFF_W1N:OFF_W1N + F] = d['w1n']
  p[OFF_B1:OFF_B1 + F] = d['b1']
  p[OFF_W2:OFF_B2] = np.asarray(d['W2']).reshape(-1)
  p[OFF_B2:OFF_B2 + F] = d['b2']
  p[OFF_W3:OFF_B3] = np.asarray(d['W3']).reshape(-1)
  p[OFF_B3:OFF_B3 + F] = d['b3']
  p[OFF_WO:OFF_WO + F] = d['wo']
  p[OFF_BO] = d['bo']
  return p


def init_params(seed=0):
  """Glorot-uniform weights, zero biases (any start works for the tests)."""
  rng = np.random.default_rng(seed)
  d = {'w1s': rng.uniform(-1, 1, F) * np.sqrt(6 / (2 + F)),
       'w1n': rng.uniform(-1, 1, F) * np.sqrt(6 / (2 + F)),
       'b1': np.zeros(F),
       'W2': rng.uniform(-1, 1, (2 * F, F)) * np.sqrt(6 / (3 * F)), 'b2': np.zeros(F),
       'W3': rng.uniform(-1, 1, (2 * F, F)) * np.sqrt(6 / (3 * F)), 'b3': np.zeros(F),
       'wo': rng.uniform(-1, 1, F) * np.sqrt(6 / (1 + F)), 'bo': 0.0}
  return pack(d).astype(np.float32)


class Graph:
  """The scaled coarse matrix Ah = S A S of a CSR matrix with 1/diag."""

  def __init__(self, indptr, indices, data, diag_inv):
    n = len(indptr) - 1
    dinv = np.asarray(diag_inv, np.float64)
    self.n = n
    self.s = np.where(dinv > 0, np.sqrt(np.maximum(dinv, 0)), 0.0)
    self.s32 = np.sqrt(np.maximum(np.asarray(diag_inv, np.float32), 0)).astype(np.float32)
    self.s32[np.asarray(diag_inv, np.float32) <= 0] = 0
    A = sp.csr_matrix((np.asarray(data, np.float64), np.asarray(indices), np.asarray(indptr)),
                      shape=(n, n))
    self.A = A
    self.Ah = sp.diags(self.s) @ A @ sp.diags(self.s)


def forward(p, g: Graph, r, device=True):
  """Returns (e_c, cache) for one restricted residual r (n,)."""
  P = unpack(p)
  rd = bf16 if device else (lambda v: v)
  W2 = rd(P['W2'].astype(np.float32)).astype(np.float64) if device else P['W2']
  W3 = rd(P['W3'].astype(np.float32)).astype(np.float64) if device else P['W3']
  s = g.s32.astype(np.float64) if device else g.s
  sr = s * np.asarray(r, np.float64)
  sigma = np.sqrt(np.sum(sr * sr) / g.n)
  if sigma == 0.0:
    return np.zeros(g.n), None
  u = sr / sigma
  a1 = g.Ah @ u
  H1 = rd(np.maximum(np.outer(u, P['w1s']) + np.outer(a1, P['w1n']) + P['b1'], 0))
  G1 = rd(g.Ah @ H1)
  H2 = rd(np.maximum(np.hstack([H1, G1]) @ W2 + P['b2'], 0))
  G2 = rd(g.Ah @ H2)
  H3 = np.maximum(np.hstack([H2, G2]) @ W3 + P['b3'], 0)
  y = H3 @ P['wo'] + P['bo']
  cache = dict(u=u, a1=a1, H1=H1, G1=G1, H2=H2, G2=G2, H3=H3, y=y, W2=W2, W3=W3, sigma=sigma)
  return sigma * s * y, cache


def energy(g: Graph, r, e):
  """1/2 e^T A e - e^T r of the unscaled coarse system."""
  e = np.asarray(e, np.float64)
  return 0.5 * e @ (g.A @ e) - e @ np.asarray(r, np.float64)


def feature_field(g: Graph):
  """r_i = sqrt(A_ii), so that u = S r / sigma = 1 (float32 like the kernels)."""
  d = np.asarray(g.s32, np.float32)
  return np.where(d > 0, (np.float32(1.0) / d).astype(np.float32), np.float32(0.0))


def weight_cap(g: Graph):
  """1.9 / sum_j |Ah_ij| per row (0 for an empty row)."""
  R = np.asarray(abs(g.Ah).sum(axis=1)).reshape(-1)
  return np.where(R > 0, 1.9 / np.where(R > 0, R, 1.0), 0.0)


def weights(p, g: Graph, device=True):
  """The per-aggregate weights w = cap * sigmoid(y), y the network on the
  feature field; also returns the cache with dw/dy ('dw')."""
  _, c = forward(p, g, feature_field(g), device)
  cap = weight_cap(g)
  sg = 1.0 / (1.0 + np.exp(-c['y']))
  w = cap * sg
  c['dw'] = cap * sg * (1.0 - sg)
  return w, c


def apply_weights(g: Graph, w, r):
  """e = max(w, 0) * r / diag(A) (the correction applied in each V-cycle;
  weights() is already non-negative)."""
  d = g.s32.astype(np.float64) ** 2
  return np.maximum(w, 0) * d * np.asarray(r, np.float64)


def _backward(P, g: Graph, c, gy, gd):
  gd['wo'] = gd.get('wo', 0) + c['H3'].T @ gy
  gd['bo'] = gd.get('bo', 0) + gy.sum()
  gZ3 = np.outer(gy, P['wo']) * (c['H3'] > 0)
  gd['W3'] = gd.get('W3', 0) + np.hstack([c['H2'], c['G2']]).T @ gZ3
  gd['b3'] = gd.get('b3', 0) + gZ3.sum(0)
  gX3 = gZ3 @ c['W3'].T
  gH2 = gX3[:, :F] + g.Ah @ gX3[:, F:]
  gZ2 = gH2 * (c['H2'] > 0)
  gd['W2'] = gd.get('W2', 0) + np.hstack([c['H1'], c['G1']]).T @ gZ2
  gd['b2'] = gd.get('b2', 0) + gZ2.sum(0)
  gX2 = gZ2 @ c['W2'].T
  gH1 = gX2[:, :F] + g.Ah @ gX2[:, F:]
  gZ1 = gH1 * (c['H1'] > 0)
  gd['w1s'] = gd.get('w1s', 0) + c['u'] @ gZ1
  gd['w1n'] = gd.get('w1n', 0) + c['a1'] @ gZ1
  gd['b1'] = gd.get('b1', 0) + gZ1.sum(0)


def _scaled(g: Graph, r, device):
  s = g.s32.astype(np.float64) if device else g.s
  sr = s * np.asarray(r, np.float64)
  sigma = np.sqrt(np.sum(sr * sr) / g.n)
  return sr / sigma if sigma > 0 else np.zeros(g.n)


def loss_and_grad(p, g: Graph, samples, device=True, mode='weights'):
  """Mean scaled energy over the samples and its gradient w.r.t. p.

  mode='weights': the correction is w * r / diag(A) with w = weights(p, g);
  mode='field': the correction is the network applied to the residual."""
  P = unpack(p)
  S = len(samples)
  gd = {}
  loss = 0.0
  if mode == 'weights':
    w, c = weights(p, g, device)
    gy = np.zeros(g.n)
    for r in samples:
      u = _scaled(g, r, device)
      v = w * u
      Av = g.Ah @ v
      loss += (0.5 * v @ Av - v @ u) / (g.n * S)
      gy += (Av - u) * u * c['dw'] / (g.n * S)
    _backward(P, g, c, gy, gd)
    return loss, pack({k: gd.get(k, 0) for k in ('w1s', 'w1n', 'b1', 'W2', 'b2', 'W3', 'b3',
                                                 'wo', 'bo')})
  for r in samples:
    _, c = forward(p, g, r, device)
    if c is None:
      continue
    y, u = c['y'], c['u']
    Ay = g.Ah @ y
    loss += (0.5 * y @ Ay - y @ u) / (g.n * S)
    _backward(P, g, c, (Ay - u) / (g.n * S), gd)
  if not gd:
    return loss, np.zeros(N_PARAMS)
  return loss, pack(gd)


def adam(p, grad, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
  """One Adam step (bias-corrected), float64; returns new (p, m, v)."""
  m = b1 * m + (1 - b1) * grad
  v = b2 * v + (1 - b2) * grad * grad
  mh = m / (1 - b1 ** t)
  vh = v / (1 - b2 ** t)
  return p - lr * mh / (np.sqrt(vh) + eps), m, v
