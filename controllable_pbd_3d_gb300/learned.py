"""Learned coarse correction for the MGPBD PCG (no counterpart in the reference).

The reference's V-cycle corrects the fine residual with `min(50, n)`
weighted-Jacobi sweeps on the coarsest level (cons/mgpcg_gpu.py:216-224)
of its two-level tet-aggregation hierarchy (cons/tet_aggregation.py:145-211).
The learned correction replaces those sweeps by a linear map,

    e_c = w * r_c / diag(A_c),   w_i = c_i sigmoid(y_i),   c_i = 1.9 / sum_j |Ah_ij|,

whose per-aggregate outputs y a 3-layer message-passing network computes
from the level-1 (aggregate) matrix A_c, once per Newton iteration.  The
bound keeps every weight below 2 / sum_j |Ah_ij|, where no mode of A_c is
over-corrected (Gershgorin), so the V-cycle stays positive definite; the
l1-Jacobi weight is 1 / sum_j |Ah_ij|.  On a node field r, with
s_i = (1/A_ii)^1/2 and Ah = S A_c S (hidden width 64):

    sigma = rms(S r),  u = S r / sigma,  a1 = Ah u
    H1 = relu(u w1s + a1 w1n + b1)
    H2 = relu([H1, Ah H1] W2 + b2),   H3 = relu([H2, Ah H2] W3 + b3)
    y = H3 wo + bo  (e = sigma S y),

and y is taken on the field r = sqrt(diag A_c) (u = 1; layer 1 sees the
row sums of Ah, the layers after it their neighbourhoods).  Being linear
in the residual, the correction keeps CG's convergence theory (a network
applied to the residual itself, `CoarseNet.forward`, is nonlinear and made
the long CG solves of stiff bodies stall).

Inference, the backward pass and Adam are CUDA kernels of libmgpbd.so
(`csrc/mpnn.cu`; dense layers on the tensor cores with bf16 weights and
activations, float32 accumulation).  Training data comes from the plain
solver itself (`MGPBDSolverGPU.record_coarse`): the restricted residuals r_c
its V-cycles see, paired with the plain coarse corrections.  The loss is the
scaled coarse energy of the correction, mean_s (1/2 v^T Ah v - v^T u_s)/n
with v = w * u_s, minimised by e_c = A_c^-1 r_c, so training needs no exact
solves and the plain correction is judged on the same scale
(`coarse_energy`).

`MGPBDSolverGPU(..., precond='learned')` with `set_coarse_net(net)` uses it
in every V-cycle, keeping the plain V-cycle as judge (first V-cycle of every
solve) and fallback (stalls).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N

N_PARAMS = N.MGPBD_NET_PARAMS


def _view(ptr, shape, dtype=torch.float32):
  from .mgpbd_gpu import device_view
  return device_view(ptr, shape, dtype)


def _s():
  return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class CoarseGraph:
  """A CSR matrix with its 1/diag in device memory: the aggregate graph."""

  def __init__(self, indptr, indices, data, diag_inv, keep=None):
    self.indptr, self.indices, self.data, self.diag_inv = indptr, indices, data, diag_inv
    self.n = int(indptr.shape[0]) - 1
    self.nnz = int(indices.shape[0])
    self._keep = keep

  @classmethod
  def from_solver(cls, solver, level=1):
    """Level `level` of an initialised MGPBDSolverGPU (a live view: values
    follow the solver's refills)."""
    A = solver._gpu_solver._gpu_As[level]
    return cls(A.indptr, A.indices, A.data, A.diag_inv, keep=solver)

  @classmethod
  def from_scipy(cls, A, device='cuda'):
    A = A.tocsr()
    ip = torch.tensor(np.asarray(A.indptr, np.int32), device=device)
    ix = torch.tensor(np.asarray(A.indices, np.int32), device=device)
    d = torch.tensor(np.asarray(A.data, np.float32), device=device)
    di = torch.empty(A.shape[0], dtype=torch.float32, device=device)
    N.check(N.lib().mgpbd_csr_diag_inv(A.shape[0], ip.data_ptr(), ix.data_ptr(), d.data_ptr(),
                                       di.data_ptr(), _s()), 'mgpbd_csr_diag_inv')
    return cls(ip, ix, d, di)

  def args(self):
    return (self.n, self.nnz, self.indptr.data_ptr(), self.indices.data_ptr(),
            self.data.data_ptr(), self.diag_inv.data_ptr())

  def spmv(self, x):
    y = torch.empty_like(x)
    N.check(N.lib().mgpbd_csr_spmv(self.n, self.indptr.data_ptr(), self.indices.data_ptr(),
                                   self.data.data_ptr(), x.data_ptr(), y.data_ptr(), _s()),
            'mgpbd_csr_spmv')
    return y

  def snapshot(self):
    """A copy whose values no longer follow the solver."""
    return CoarseGraph(self.indptr.clone(), self.indices.clone(), self.data.clone(),
                       self.diag_inv.clone())


def coarse_energy(graph: CoarseGraph, r, e):
  """1/2 e^T A_c e - e^T r per row of r, e (float64 on the device); lower is
  closer to A_c^-1 r in the energy norm."""
  r2 = r.reshape(-1, graph.n)
  e2 = e.reshape(-1, graph.n)
  out = []
  for rk, ek in zip(r2, e2):
    ae = graph.spmv(ek.contiguous())
    out.append(0.5 * torch.dot(ek.double(), ae.double()) - torch.dot(ek.double(), rk.double()))
  return torch.stack(out)


class CoarseNet:
  """The network's parameters (device float32) and its CUDA entry points."""

  def __init__(self, seed: int = 0):
    self._lib = N.lib()
    h = C.c_void_p()
    N.check(self._lib.mgpbd_net_create(C.c_uint64(seed), C.byref(h)), 'mgpbd_net_create')
    self._h = h
    p, g = C.c_void_p(), C.c_void_p()
    N.check(self._lib.mgpbd_net_params(h, C.byref(p), C.byref(g)), 'mgpbd_net_params')
    self.params = _view(p.value, (N_PARAMS,))
    self.grad = _view(g.value, (N_PARAMS,))

  def __del__(self):
    h = getattr(self, '_h', None)
    if h is not None and h.value:
      try:
        self._lib.mgpbd_net_destroy(h)
      except Exception:
        pass
      self._h = None

  def load_params(self, p):
    self.params.copy_(torch.as_tensor(np.asarray(p, np.float32)).to(self.params.device))
    N.check(self._lib.mgpbd_net_sync_params(self._h, _s()), 'mgpbd_net_sync_params')

  def state(self) -> np.ndarray:
    return self.params.detach().cpu().numpy().copy()

  def forward(self, graph: CoarseGraph, r):
    """The network on the field r (n,) or on each row of (S, n)."""
    r = r.contiguous()
    e = torch.empty_like(r)
    for rk, ek in zip(r.reshape(-1, graph.n), e.reshape(-1, graph.n)):
      N.check(self._lib.mgpbd_net_forward(self._h, *graph.args(), rk.data_ptr(), ek.data_ptr(),
                                          _s()), 'mgpbd_net_forward')
    return e

  def weights(self, graph: CoarseGraph):
    """The per-aggregate weights w of the graph."""
    w = torch.empty(graph.n, dtype=torch.float32, device=graph.data.device)
    N.check(self._lib.mgpbd_net_weights(self._h, *graph.args(), w.data_ptr(), _s()),
            'mgpbd_net_weights')
    return w

  def correction(self, graph: CoarseGraph, r, w=None):
    """e_c = w * r / diag(A_c) for residuals r (n,) or (S, n)."""
    if w is None:
      w = self.weights(graph)
    r = r.contiguous()
    e = torch.empty_like(r)
    for rk, ek in zip(r.reshape(-1, graph.n), e.reshape(-1, graph.n)):
      N.check(self._lib.mgpbd_net_apply(graph.n, w.data_ptr(), graph.diag_inv.data_ptr(),
                                        rk.data_ptr(), ek.data_ptr(), _s()), 'mgpbd_net_apply')
    return e

  def loss_grad(self, graph: CoarseGraph, samples, mode='weights') -> float:
    """Mean scaled coarse energy of the batch; the gradient lands in .grad.
    mode='weights': of the correction w * r / diag(A); 'field': of the
    network applied to each residual."""
    samples = samples.contiguous()
    loss = C.c_double()
    m = {'weights': N.MGPBD_NET_LOSS_WEIGHTS, 'field': N.MGPBD_NET_LOSS_FIELD}[mode]
    N.check(self._lib.mgpbd_net_loss_grad(self._h, *graph.args(), samples.data_ptr(),
                                          samples.shape[0], m, C.byref(loss), _s()),
            'mgpbd_net_loss_grad')
    return loss.value

  def adam_step(self, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
    N.check(self._lib.mgpbd_net_adam(self._h, float(lr), float(betas[0]), float(betas[1]),
                                     float(eps), _s()), 'mgpbd_net_adam')

  def fit(self, graph: CoarseGraph, samples, steps=200, batch=8, lr=1e-3) -> np.ndarray:
    """`steps` Adam steps (weights loss) on batches of `batch` residuals;
    returns the losses."""
    samples = samples.contiguous()
    losses = np.zeros(max(int(steps), 1), np.float64)
    N.check(self._lib.mgpbd_net_train(self._h, *graph.args(), samples.data_ptr(),
                                      samples.shape[0], int(batch), int(steps), float(lr),
                                      losses.ctypes.data, _s()), 'mgpbd_net_train')
    return losses[:int(steps)]

  def fit_many(self, data, steps=200, batch=8, lr=1e-3) -> np.ndarray:
    """Alternate Adam steps over several (graph, samples) pairs (different
    bodies); the weights are shared, the graphs differ."""
    out = []
    data = [(g, s.contiguous()) for g, s in data]
    offs = [0] * len(data)
    for k in range(int(steps)):
      j = k % len(data)
      g, s = data[j]
      idx = [(offs[j] + i) % s.shape[0] for i in range(batch)]
      offs[j] = (offs[j] + batch) % s.shape[0]
      out.append(self.loss_grad(g, s[idx]))
      self.adam_step(lr)
    return np.asarray(out)



# the plain solver that produces training pairs: the reference's V-cycle PCG
# on CSR (parity mode) with the capped smoother weight, one Newton iteration
PAIR_SOLVER_KW = dict(mode='parity', smoother='safe', precond='vcycle', damp=1.0, maxiter=1,
                      maxiter_cg=6000, tol_cg=1e-12, rel_tol_cg=1e-6, n_smooth=2,
                      kinematic_pins=True)


def collect_pairs(body, n_pairs=64, every=4, constraints='edge_volume', dt=1.0 / 300.0,
                  device='cuda', cg_limit=None):
  """Training pairs of one body (a dict of `scenarios.training_body`): one
  Newton iteration of the plain solver, recording up to `n_pairs`
  restricted residuals r_c (every `every`-th V-cycle); returns the level-1
  graph (a snapshot that outlives the solver) and the (k, n1) residuals.
  cg_limit: stop the solve after that many CG iterations (the pairs come
  from its first n_pairs * every V-cycles)."""
  from .mgpbd_gpu import MGPBDSolverGPU
  x = torch.tensor(body['x0'], device=device)
  s = MGPBDSolverGPU(x, torch.tensor(body['x_ref'], device=device),
                     torch.tensor(body['invm'], device=device),
                     torch.tensor(body['t_i'], device=device), None, [0.0, -9.8, 0.0], dt,
                     compliance=float(body['compliance']), constraints=constraints,
                     **dict(PAIR_SOLVER_KW, **({} if cg_limit is None else
                                               {'maxiter_cg': int(cg_limit)})))
  s.init()
  s.record_coarse(int(n_pairs), int(every))
  s.step(0)
  rc, _ = s.recorded_coarse()
  g = s.coarse_graph().snapshot()
  rc = rc.clone()
  del s
  return g, rc


def train_on_bodies(net: CoarseNet, bodies, pairs_per_body=64, every=4, steps=600, batch=8,
                    lr=2e-3, constraints='edge_volume', cg_limit=None):
  """Train `net` on pairs from several bodies (an iterable of
  `scenarios.training_body` dicts): pairs are collected body by body, then
  `fit_many` alternates Adam steps over the bodies.  Returns
  (losses, [(graph, residuals)])."""
  data = []
  for b in bodies:
    g, rc = collect_pairs(b, pairs_per_body, every, constraints, cg_limit=cg_limit)
    if rc.shape[0] > 0:
      data.append((g, rc))
  if not data:
    raise RuntimeError('no training pairs recorded (every solve converged before the '
                       'first recorded V-cycle)')
  return net.fit_many(data, steps=steps, batch=batch, lr=lr), data
