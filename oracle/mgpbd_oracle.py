"""CPU restatement of the reference's MGPBD GPU step, for checking only.

TEST INFRASTRUCTURE: this module is the oracle the CUDA path is compared
against.  It is imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, never by the product package.

It restates, in vectorised numpy/scipy and in the arithmetic type chosen
(`np.float32` = the reference's precision, `np.float64` = exact-arithmetic
stand-in), the algorithm of:

* cons/mgpbd_gpu.py:136-151  rest shape (Dm^-1, volume, alpha~ = 1/(mu dt^2 V))
* cons/mgpbd_gpu.py:153-194  level-0 CSR pattern, sorted neighbours + diagonal last
* cons/mgpbd_gpu.py:206-219  prediction / velocity update
* cons/mgpbd_gpu.py:225-247 and cons/mgpbd.py:35-68  ARAP C = |S - I| and grad C
* cons/mgpbd_gpu.py:253-267  b = -(C + alpha~ lambda), |b|
* cons/mgpbd_gpu.py:273-309 and cons/mgpbd.py:72-84  A = J W J^T + alpha~
* cons/mgpbd_gpu.py:330-391  scatter, apply, backtracking line search
* cons/mgpbd_gpu.py:397-446  the Newton loop
* cons/tet_aggregation.py:11-211  face adjacency, greedy aggregation, hierarchy
* cons/mgpcg_gpu.py:43-99     Galerkin RAP pattern (scipy) + contribution map
* cons/mgpcg_gpu.py:183-329   coarse refill, V-cycle, PCG with its guards
* cons/sparse_gpu.py:18-144   CSR spmv, weighted Jacobi, 1/diag

One deliberate deviation, shared with the CUDA path: the level-0 matrix keeps
the diagonal-last column order for both values and indices (the reference's
GPU setup sorts the indices but not the values it writes later; see
tests/golden/make_golden.py).

Pinned by tests/golden/*.npz, which were produced by running the reference's
own Python code (Taichi replaced by a numpy shim); see tests/test_oracle.py.
The extra solver options (`smoother='safe'`, `coarse='dense'`,
`rel_tol_cg`, `extra_levels`, `kinematic_pins`) mirror the FAST-mode options of
the CUDA library and have no reference counterpart.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

# ----------------------------------------------------------------------------
# structure (integer, bit-exact)
# ----------------------------------------------------------------------------


def sparsity_pattern(t_i, nt):
  """cons/mgpbd_gpu.py:153-194: row t = sorted vertex-sharing tets, then t."""
  t = np.asarray(t_i, np.int64).reshape(nt, 4)
  nv = int(t.max()) + 1
  inc = sp.csr_matrix((np.ones(4 * nt), (np.repeat(np.arange(nt), 4), t.reshape(-1))),
                      shape=(nt, nv))
  s = (inc @ inc.T).tocsr()
  s.sort_indices()
  rows = np.repeat(np.arange(nt), np.diff(s.indptr))
  keep = s.indices != rows
  cols = s.indices[keep]
  r = rows[keep]
  counts = np.bincount(r, minlength=nt) + 1
  indptr = np.zeros(nt + 1, np.int64)
  indptr[1:] = np.cumsum(counts)
  indices = np.empty(indptr[-1], np.int64)
  # off-diagonal block of row i goes to [indptr[i], indptr[i+1]-1)
  off_start = indptr[:-1]
  pos = off_start[r] + (np.arange(len(r)) - np.searchsorted(r, r, side='left'))
  indices[pos] = cols
  indices[indptr[1:] - 1] = np.arange(nt)
  return indptr.astype(np.int32), indices.astype(np.int32)


def face_adjacency_sets(t_i, nt):
  """cons/tet_aggregation.py:11-37 with Python sets filled in the same order
  (faces in first-appearance order), so set iteration order matches."""
  t = np.asarray(t_i).reshape(nt, 4).tolist()
  face_to = {}
  for k in range(nt):
    v = t[k]
    for skip in range(4):
      f = tuple(sorted(v[j] for j in range(4) if j != skip))
      lst = face_to.get(f)
      if lst is None:
        face_to[f] = [k]
      else:
        lst.append(k)
  adj = [set() for _ in range(nt)]
  for lst in face_to.values():
    if len(lst) == 2:
      adj[lst[0]].add(lst[1])
      adj[lst[1]].add(lst[0])
  return adj


def tet_aggregation(t_i, nt, max_agg_size=8):
  """cons/tet_aggregation.py:40-127 (pass 1; pass 2 never triggers).

  The candidate set is built the way CPython builds `adj[seed] - visited`
  when `visited` is the larger set: a new set filled by iterating
  `adj[seed]` and keeping the unvisited ids, which gives the same iteration
  order as the reference."""
  adj = face_adjacency_sets(t_i, nt)
  deg = [len(a) for a in adj]
  order = sorted(range(nt), key=lambda k: deg[k])
  agg = np.full(nt, -1, np.int32)
  visited = bytearray(nt)
  n_visited = 0
  n_agg = 0
  for seed in order:
    if visited[seed]:
      continue
    agg[seed] = n_agg
    visited[seed] = 1
    n_visited += 1
    size = 1
    so = adj[seed]
    if (len(so) >> 2) > n_visited:
      diff = set(so)
      for k in so:
        if visited[k]:
          diff.discard(k)
    else:
      diff = set()
      for k in so:
        if not visited[k]:
          diff.add(k)
    cand = sorted(diff, key=lambda k: deg[k])
    for nb in cand:
      if visited[nb]:
        continue
      if size >= max_agg_size:
        break
      agg[nb] = n_agg
      visited[nb] = 1
      n_visited += 1
      size += 1
      if size < max_agg_size:
        for nb2 in adj[nb]:
          if not visited[nb2] and size < max_agg_size:
            agg[nb2] = n_agg
            visited[nb2] = 1
            n_visited += 1
            size += 1
    n_agg += 1
  return agg, n_agg


def tet_hierarchy(t_i, nt, max_coarse=400, max_levels=4):
  """cons/tet_aggregation.py:145-211: (list of agg arrays, sizes)."""
  sizes = [nt]
  aggs = []
  cur = np.asarray(t_i, np.int32).reshape(-1)
  cur_nt = nt
  for _ in range(max_levels):
    if cur_nt <= max_coarse:
      break
    max_agg = max(min(8, max(2, cur_nt // max(max_coarse, 1))), 2)
    agg, n_agg = tet_aggregation(cur, cur_nt, max_agg)
    if n_agg >= cur_nt:
      break
    aggs.append(agg)
    sizes.append(n_agg)
    cur = np.repeat(np.arange(n_agg, dtype=np.int32), 4)
    cur_nt = n_agg
  return aggs, sizes


def galerkin(indptr, indices, data, agg, n_agg, by_value=True):
  """cons/mgpcg_gpu.py:43-99 for piecewise-constant P.

  The coarse pattern is scipy's (P^T A) P in float64 (exact zeros dropped,
  sorted columns); the contribution map lists, per coarse entry, the fine
  entries in (member row ascending, stored position) order.  With
  `by_value=False` the structural pattern (no value-based dropping) is used.
  """
  n = len(indptr) - 1
  vals = np.asarray(data, np.float64) if by_value else np.ones(len(indices))
  a = sp.csr_matrix((vals, np.asarray(indices), np.asarray(indptr)), shape=(n, n))
  P = sp.csr_matrix((np.ones(n), (np.arange(n), np.asarray(agg))), shape=(n, n_agg))
  ac = (P.T @ a @ P).tocsr()
  ac.sort_indices()
  c_indptr = ac.indptr.astype(np.int64)
  c_indices = ac.indices.astype(np.int64)
  rows = np.repeat(np.arange(n), np.diff(indptr))
  I = np.asarray(agg)[rows]
  J = np.asarray(agg)[np.asarray(indices)]
  # coarse position of (I, J), -1 if dropped
  key_c = np.repeat(np.arange(n_agg), np.diff(c_indptr)) * n_agg + c_indices
  key_f = I.astype(np.int64) * n_agg + J
  pos = np.searchsorted(key_c, key_f)
  pos = np.minimum(pos, len(key_c) - 1)
  hit = key_c[pos] == key_f
  c = np.where(hit, pos, -1)
  sel = np.nonzero(c >= 0)[0]
  order = sel[np.argsort(c[sel], kind='stable')]
  counts = np.bincount(c[sel], minlength=len(c_indices))
  off = np.zeros(len(c_indices) + 1, np.int64)
  off[1:] = np.cumsum(counts)
  diag_pos = np.full(n_agg, -1, np.int64)
  rr = np.repeat(np.arange(n_agg), np.diff(c_indptr))
  d = np.nonzero(c_indices == rr)[0]
  diag_pos[rr[d]] = d
  return (c_indptr.astype(np.int32), c_indices.astype(np.int32), order.astype(np.int32),
          off.astype(np.int32), diag_pos)


def graph_aggregate(indptr, indices, max_agg_size=8):
  """Greedy matrix-graph aggregation (the CUDA library's extra levels; no
  reference counterpart)."""
  n = len(indptr) - 1
  agg = np.full(n, -1, np.int64)
  n_agg = 0
  for i in range(n):
    if agg[i] >= 0:
      continue
    nb = indices[indptr[i]:indptr[i + 1]]
    if np.any(agg[nb] >= 0):
      continue
    size = 0
    for j in nb:
      if size >= max_agg_size:
        break
      if agg[j] < 0:
        agg[j] = n_agg
        size += 1
    if agg[i] < 0:
      agg[i] = n_agg
    n_agg += 1
  for i in range(n):
    if agg[i] >= 0:
      continue
    for j in indices[indptr[i]:indptr[i + 1]]:
      if j != i and agg[j] >= 0:
        agg[i] = agg[j]
        break
    if agg[i] < 0:
      agg[i] = n_agg
      n_agg += 1
  return agg.astype(np.int32), n_agg


def edge_volume_system(t_i):
  """The length + volume constraint set of a tet mesh, restated for the
  oracle: one volume constraint per tet (slots v0..v3, C = det F - 1 as in
  cons/deform3d.py:81-83), then one length constraint per unique tet edge
  (a < b, edges in ascending (a, b) order; slots a, b, a, b; C = |x_a - x_b|
  - L0 as in cons/length.py:65-90).  Returns (c_i, ctype, edges, owner),
  owner = the lowest-numbered tet containing the edge."""
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  nt = len(t)
  nv = int(t.max()) + 1
  pairs = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
  a = np.concatenate([np.minimum(t[:, i], t[:, j]) for i, j in pairs])
  b = np.concatenate([np.maximum(t[:, i], t[:, j]) for i, j in pairs])
  tet = np.tile(np.arange(nt), len(pairs))
  key = a * nv + b
  uniq, inv = np.unique(key, return_inverse=True)
  owner = np.full(len(uniq), nt, np.int64)
  np.minimum.at(owner, inv, tet)
  edges = np.stack([uniq // nv, uniq % nv], 1)
  c = np.concatenate([t, edges[:, [0, 1, 0, 1]]]).astype(np.int32)
  ctype = np.concatenate([np.full(nt, CONS_VOLUME), np.full(len(edges), CONS_LENGTH)])
  return c.reshape(-1), ctype.astype(np.int32), edges.astype(np.int32), owner.astype(np.int32)


def edge_volume_hierarchy(t_i, max_coarse=400):
  """Level-0 aggregates of the length + volume constraints from the
  reference's tet aggregation (cons/tet_aggregation.py:145-211): a volume
  constraint lies in its tet's aggregate, a length constraint in its owner
  tet's.  Returns (aggs, sizes) as tet_hierarchy does, one level."""
  t = np.asarray(t_i, np.int32).reshape(-1)
  nt = len(t) // 4
  aggs, sizes = tet_hierarchy(t, nt, max_coarse)
  if not aggs:
    return [], [nt]
  _, _, edges, owner = edge_volume_system(t)
  agg_t = np.asarray(aggs[0], np.int64)
  return [np.concatenate([agg_t, agg_t[owner]]).astype(np.int32)], [nt + len(edges), sizes[1]]


# ----------------------------------------------------------------------------
# per-tet / per-vertex arithmetic
# ----------------------------------------------------------------------------


CONS_ARAP, CONS_LENGTH, CONS_VOLUME = 0, 1, 2


def rest_shape(x_ref, t_i, mu, dt, dtype=np.float32, compliance=0.0, ctype=None):
  """cons/mgpbd_gpu.py:136-151 (compliance > 0: alpha~ = compliance / dt^2).

  With constraint types (the library's MGPBD_CONS_*), a length constraint
  (slots a, b, a, b) gets its rest length in the volume's place and no
  Dm^-1 (zeros)."""
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  x = np.asarray(x_ref, dtype)
  nt = len(t)
  is_len = np.zeros(nt, bool) if ctype is None else np.asarray(ctype) == CONS_LENGTH
  Dm = np.stack([x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]], x[t[:, 3]] - x[t[:, 0]]], axis=2)
  dm_inv = np.zeros((nt, 3, 3), dtype)
  vol = np.zeros(nt, dtype)
  tt = ~is_len
  dm_inv[tt] = np.linalg.inv(Dm[tt].astype(np.float64)).astype(dtype)
  vol[tt] = (np.abs(np.linalg.det(Dm[tt].astype(np.float64))) / 6.0).astype(dtype)
  d = (x[t[is_len, 0]] - x[t[is_len, 1]]).astype(np.float64)
  vol[is_len] = np.sqrt((d * d).sum(axis=1)).astype(dtype)
  if compliance > 0:
    alpha = np.full(nt, dtype(compliance) / (dtype(dt) * dtype(dt)), dtype)
  else:
    alpha = (dtype(1.0) / (dtype(mu) * dtype(dt) * dtype(dt) * vol)).astype(dtype)
  return dm_inv, vol, alpha


def volume_values(F):
  """det F - 1 and d(det F)/dF (columns f2 x f3, f3 x f1, f1 x f2): the
  hydrostatic constraint of cons/deform3d.py:81-83."""
  f1, f2, f3 = F[:, :, 0], F[:, :, 1], F[:, :, 2]
  P = np.stack([np.cross(f2, f3), np.cross(f3, f1), np.cross(f1, f2)], axis=2)
  return (f1 * P[:, :, 0]).sum(axis=1) - 1.0, P


def length_values(x, t_i, rest, dtype):
  """|x_a - x_b| - L0 and the unit vector a - b (cons/length.py:65-90)."""
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  x = np.asarray(x, dtype)
  d = x[t[:, 0]] - x[t[:, 1]]
  ln = np.sqrt((d.astype(np.float64) ** 2).sum(axis=1))
  n = np.where(ln[:, None] > 1e-12, d / np.where(ln > 0, ln, 1.0)[:, None], 0.0)
  return (ln - np.asarray(rest, np.float64)).astype(dtype), n.astype(dtype)


def svd_rv(F):
  """Rotation-variant SVD (det U = det V = +1, sign of det F on s[2]),
  computed in float64."""
  A = np.asarray(F, np.float64)
  u, s, vt = np.linalg.svd(A)
  v = np.swapaxes(vt, -1, -2).copy()
  u = u.copy()
  s = s.copy()
  nu = np.linalg.det(u) < 0
  u[nu, :, 2] *= -1.0
  s[nu, 2] *= -1.0
  nv_ = np.linalg.det(v) < 0
  v[nv_, :, 2] *= -1.0
  s[nv_, 2] *= -1.0
  return u, s, v


def deformation(x, t_i, dm_inv, dtype):
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  x = np.asarray(x, dtype)
  Ds = np.stack([x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]], x[t[:, 3]] - x[t[:, 0]]], axis=2)
  return Ds @ np.asarray(dm_inv, dtype)


def constraint_values(x, t_i, dm_inv, dtype=np.float32, ctype=None, rest=None):
  F = deformation(x, t_i, dm_inv, dtype)
  _, s, _ = svd_rv(F)
  s = s.astype(dtype)
  c = np.sqrt(((s - dtype(1.0)) ** 2).sum(axis=1)).astype(dtype)
  if ctype is not None:
    ct = np.asarray(ctype)
    vol, _ = volume_values(F.astype(np.float64))
    c = np.where(ct == CONS_VOLUME, vol.astype(dtype), c)
    ln, _ = length_values(x, t_i, rest, dtype)
    c = np.where(ct == CONS_LENGTH, ln, c).astype(dtype)
  return c


def constraints(x, t_i, dm_inv, dtype=np.float32, ctype=None, rest=None):
  """cons/mgpbd_gpu.py:225-247 + _arap_gradient (cons/mgpbd.py:35-68).

  Returns C (nt,) and gradC (nt, 4, 3): g_k = U diag((S-1)/C) V^T Dm^-T
  column k-1 for k = 1..3, g_0 = -(g_1 + g_2 + g_3), zero when C <= 1e-6.
  With constraint types: volume rows use C = det F - 1 with P = d(det F)/dF
  in place of U diag((S-1)/C) V^T; length rows C = |x_a - x_b| - L0 with
  gradients n, -n on slots 0, 1 (rest: the rest lengths)."""
  F = deformation(x, t_i, dm_inv, dtype)
  u, s, v = svd_rv(F)
  u, s, v = u.astype(dtype), s.astype(dtype), v.astype(dtype)
  C = np.sqrt(((s - dtype(1.0)) ** 2).sum(axis=1)).astype(dtype)
  ok = C > dtype(1e-6)
  Cs = np.where(ok, C, dtype(1.0))
  d = (s - dtype(1.0)) / Cs[:, None]
  P = np.einsum('nrm,nm,ncm->nrc', u, d, v).astype(dtype)
  if ctype is not None:
    ct = np.asarray(ctype)
    vol, Pv = volume_values(F.astype(np.float64))
    isv = ct == CONS_VOLUME
    P[isv] = Pv[isv].astype(dtype)
    C[isv] = vol[isv].astype(dtype)
    ok = ok | isv
  G = P @ np.swapaxes(np.asarray(dm_inv, dtype), 1, 2)
  g = np.zeros((len(C), 4, 3), dtype)
  g[:, 1:, :] = np.swapaxes(G, 1, 2)
  g[:, 0, :] = -(g[:, 1, :] + g[:, 2, :] + g[:, 3, :])
  g[~ok] = 0
  if ctype is not None:
    isl = np.asarray(ctype) == CONS_LENGTH
    ln, n = length_values(x, t_i, rest, dtype)
    C[isl] = ln[isl]
    g[isl] = 0
    g[isl, 0] = n[isl]
    g[isl, 1] = -n[isl]
  return C, g


def fill_A(indptr, indices, t_i, invm, gradC, alpha, dtype=np.float32, chunk=1 << 20):
  """cons/mgpbd_gpu.py:273-309 on the diagonal-last pattern."""
  t = np.asarray(t_i, np.int64).reshape(-1, 4)
  nt = len(t)
  w = np.asarray(invm, dtype)
  g = np.asarray(gradC, dtype)
  indptr = np.asarray(indptr, np.int64)
  indices = np.asarray(indices, np.int64)
  nnz = indptr[-1]
  data = np.empty(nnz, dtype)
  rows = np.repeat(np.arange(nt), np.diff(indptr))
  for s0 in range(0, nnz, chunk):
    s1 = min(nnz, s0 + chunk)
    i = rows[s0:s1]
    j = indices[s0:s1]
    vi = t[i]
    vj = t[j]
    eq = vi[:, :, None] == vj[:, None, :]
    dots = np.einsum('nad,nbd->nab', g[i], g[j]).astype(dtype)
    contrib = np.where(eq, w[vi][:, :, None] * dots, dtype(0.0))
    data[s0:s1] = contrib.reshape(len(i), 16).sum(axis=1, dtype=dtype)
  diag = (w[t] * (g * g).sum(axis=2)).sum(axis=1, dtype=dtype) + np.asarray(alpha, dtype)
  data[indptr[1:] - 1] = diag
  return data


def diag_inv_of(indptr, indices, data, dtype):
  n = len(indptr) - 1
  rows = np.repeat(np.arange(n), np.diff(indptr))
  d = np.zeros(n, dtype)
  m = np.asarray(indices) == rows
  d[rows[m]] = np.asarray(data)[m]
  out = np.zeros(n, dtype)
  nz = np.abs(d) > 1e-30
  out[nz] = dtype(1.0) / d[nz]
  return out


# ----------------------------------------------------------------------------
# the solver
# ----------------------------------------------------------------------------


class Level:

  def __init__(self, indptr, indices, dtype):
    self.indptr = np.asarray(indptr, np.int32)
    self.indices = np.asarray(indices, np.int32)
    self.n = len(indptr) - 1
    self.data = np.zeros(len(indices), dtype)
    self.dinv = np.zeros(self.n, dtype)
    self.omega = None
    self.agg = None  # -> next level
    self.contrib_idx = None  # from previous level
    self.contrib_off = None
    self.diag_pos = None

  def matrix(self):
    return sp.csr_matrix((self.data, self.indices, self.indptr), shape=(self.n, self.n))


class MGPBDOracle:
  """The reference MGPBD step on the CPU (see module docstring).

  Arrays: x0, x_ref (nv,3); invm (nv,); t_i (4*nt,).  Options mirror the
  reference constructor (cons/mgpbd_gpu.py:22-42) plus the CUDA library's
  extensions."""

  def __init__(self, x0, x_ref, invm, t_i, gravity, dt, mu=1e6, damp=1.0, maxiter=20, atol=1e-4,
               rtol=1e-2, maxiter_cg=100, tol_cg=1e-5, n_smooth=2, omega_jacobi=2.0 / 3.0,
               use_line_search=True, dtype=np.float32, kinematic_pins=False, rel_tol_cg=0.0,
               smoother='jacobi', coarse='jacobi', extra_levels=0, max_coarse=400,
               coarse_sweeps=0, hierarchy=None, cg_alias=False, compliance=0.0, ctype=None,
               linear='pcg', exact_tol=1e-11, warm_substep=False):
    """linear='pcg': the reference's V-cycle PCG; 'exact': each Newton
    system solved to a float64 dual residual of exact_tol |b|
    (oracle/exact_solve.py), for checking positions against the step with
    an exact linear solve; 'cheb': the library's FAST linear solve (CG
    with a Chebyshev-8 polynomial in A, lo 1e-3, to rel_tol_cg) in float64,
    the same algorithm as the CUDA path in exact arithmetic's stead (both
    float64 only); warm_substep (with 'cheb'): each substep's first solve
    starts from the previous substep's first solution, as the library's
    warm_substep option does."""
    if linear not in ('pcg', 'exact', 'cheb'):
      raise ValueError("linear must be 'pcg', 'exact' or 'cheb'")
    if linear != 'pcg' and dtype != np.float64:
      raise ValueError(f"linear='{linear}' is a float64 oracle")
    self.linear = linear
    self.exact_tol = exact_tol
    self.warm_substep = bool(warm_substep)
    self.dlam_prev = None
    self.exact_log = []
    self.dtype = dtype
    f = dtype
    self.x = np.array(x0, f).reshape(-1, 3)
    self.x_ref = np.array(x_ref, f).reshape(-1, 3)
    self.invm = np.array(invm, f)
    self.t_i = np.asarray(t_i, np.int32).reshape(-1)
    self.nv = len(self.x)
    self.nt = len(self.t_i) // 4
    self.g = np.asarray(gravity, f)
    self.dt = f(dt)
    self.mu = mu
    self.damp = f(damp)
    self.maxiter = maxiter
    self.atol = atol
    self.rtol = rtol
    self.maxiter_cg = maxiter_cg
    self.tol_cg = tol_cg
    self.n_smooth = n_smooth
    self.omega = f(omega_jacobi)
    self.use_line_search = use_line_search
    self.kinematic = kinematic_pins
    self.rel_tol_cg = rel_tol_cg
    self.smoother = smoother
    self.coarse = coarse
    self.extra_levels = extra_levels
    self.max_coarse = max_coarse
    self.coarse_sweeps = coarse_sweeps
    self._hierarchy = hierarchy
    self.cg_alias = cg_alias
    self.compliance = compliance
    self.ctype = None if ctype is None else np.asarray(ctype, np.int32)
    self._vres = None
    self.v = np.zeros_like(self.x)
    self.x_old = np.zeros_like(self.x)
    self.log = []

  # cons/mgpbd_gpu.py:92-114
  def init(self):
    f = self.dtype
    self.dm_inv, self.rest_vol, self.alpha = rest_shape(self.x_ref, self.t_i, self.mu, float(self.dt), f,
                                                        self.compliance, self.ctype)
    self.lam = np.zeros(self.nt, f)
    self.C, self.gradC = constraints(self.x, self.t_i, self.dm_inv, f, self.ctype, self.rest_vol)
    if self.linear != 'pcg':
      self.levels = []  # no assembled matrix: these solves are matrix-free in A
      return
    ip, ix = sparsity_pattern(self.t_i, self.nt)
    L0 = Level(ip, ix, f)
    self.levels = [L0]
    L0.data = fill_A(ip, ix, self.t_i, self.invm, self.gradC, self.alpha, f)
    if self._hierarchy is None:
      aggs, sizes = tet_hierarchy(self.t_i, self.nt, self.max_coarse)
    else:
      aggs, sizes = self._hierarchy
    vals = L0.data
    for l, agg in enumerate(aggs):
      F = self.levels[l]
      ci, cx, cidx, coff, dpos = galerkin(F.indptr, F.indices, vals, agg, sizes[l + 1])
      F.agg = np.asarray(agg, np.int64)
      Cl = Level(ci, cx, f)
      Cl.contrib_idx, Cl.contrib_off, Cl.diag_pos = cidx, coff, dpos
      Cl.data = self._refill(vals, Cl)
      vals = Cl.data
      self.levels.append(Cl)
    extra = 0
    while extra < self.extra_levels and self.levels[-1].n > self.max_coarse:
      F = self.levels[-1]
      agg, n_agg = graph_aggregate(F.indptr, F.indices, 8)
      if n_agg >= F.n:
        break
      ci, cx, cidx, coff, dpos = galerkin(F.indptr, F.indices, F.data, agg, n_agg, by_value=False)
      F.agg = np.asarray(agg, np.int64)
      Cl = Level(ci, cx, f)
      Cl.contrib_idx, Cl.contrib_off, Cl.diag_pos = cidx, coff, dpos
      self.levels.append(Cl)
      extra += 1

  def _refill(self, fine, Cl):
    f = self.dtype
    vals = np.asarray(fine, f)[Cl.contrib_idx]
    out = np.zeros(len(Cl.indices), f)
    nz = np.diff(Cl.contrib_off) > 0
    if vals.size:
      sums = np.add.reduceat(vals, Cl.contrib_off[:-1][nz]) if nz.any() else np.zeros(0, f)
      out[nz] = sums
    return out

  # cons/mgpbd_gpu.py:206-219
  def make_prediction(self):
    f = self.dtype
    self.x_old = self.x.copy()
    mov = np.ones(self.nv, bool) if not self.kinematic else self.invm != 0
    v = (self.v + self.dt * self.g) * self.damp
    self.v[mov] = v[mov]
    self.x[mov] = (self.x + self.dt * self.v).astype(f)[mov]

  def update_vel(self):
    self.v = (self.damp * (self.x - self.x_old) / self.dt).astype(self.dtype)

  def step(self, frame=0):
    self.make_prediction()
    self.solve(frame)
    self.update_vel()

  # _fill_A_and_update_gpu (cons/mgpbd_gpu.py:320-324)
  def fill_matrices(self):
    f = self.dtype
    L0 = self.levels[0]
    L0.data = fill_A(L0.indptr, L0.indices, self.t_i, self.invm, self.gradC, self.alpha, f)
    L0.dinv = diag_inv_of(L0.indptr, L0.indices, L0.data, f)
    for l in range(1, len(self.levels)):
      Cl = self.levels[l]
      Cl.data = self._refill(self.levels[l - 1].data, Cl)
      Cl.dinv = diag_inv_of(Cl.indptr, Cl.indices, Cl.data, f)
    for L in self.levels:
      L.omega = self.omega
    if self.smoother == 'safe':
      for L in self.levels:
        L.omega = f(min(float(self.omega), 4.0 / (3.0 * 1.1 * self._lambda_max(L))))
    if self.coarse == 'dense':
      A = self.levels[-1].matrix().toarray().astype(np.float64)
      self._chol = np.linalg.cholesky(A)

  def _lambda_max(self, L):
    A = L.matrix().astype(np.float64)
    d = np.asarray(L.dinv, np.float64)
    w = np.linalg.eigvals((A.toarray() * d[:, None])) if L.n <= 2000 else None
    if w is not None:
      return float(np.max(w.real))
    v = np.ones(L.n)
    lam = 1.0
    for _ in range(50):
      y = d * (A @ v)
      lam = np.linalg.norm(y) / np.linalg.norm(v)
      v = y / np.linalg.norm(y)
    return lam

  # GPUSparseMatrix.jacobi_smooth + gpu_copy (cons/sparse_gpu.py:134-144)
  def _jacobi(self, L, b, x):
    f = self.dtype
    ax = (L.matrix() @ x).astype(f)
    return (x + (L.omega * L.dinv) * (b - ax)).astype(f)

  # GPUMultigridSolver.vcycle (cons/mgpcg_gpu.py:214-259), zero initial guess
  def vcycle(self, l, b):
    f = self.dtype
    L = self.levels[l]
    x = np.zeros(L.n, f)
    if l == len(self.levels) - 1:
      if self.coarse == 'dense':
        y = np.linalg.solve(self._chol, np.asarray(b, np.float64))
        return np.linalg.solve(self._chol.T, y).astype(f)
      sweeps = self.coarse_sweeps if self.coarse_sweeps > 0 else min(50, L.n)
      for _ in range(sweeps):
        x = self._jacobi(L, b, x)
      return x
    for _ in range(self.n_smooth):
      x = self._jacobi(L, b, x)
    r = (b - (L.matrix() @ x).astype(f)).astype(f)
    if l == 0:
      self._vres = r
    bc = np.zeros(self.levels[l + 1].n, f)
    np.add.at(bc, L.agg, r)
    xc = self.vcycle(l + 1, bc)
    x = (x + xc[L.agg]).astype(f)
    for _ in range(self.n_smooth):
      x = self._jacobi(L, b, x)
    return x

  # GPUMultigridSolver.solve (cons/mgpcg_gpu.py:261-329); scalars in float64
  def pcg(self, b):
    f = self.dtype
    A = self.levels[0].matrix()
    n = len(b)
    x = np.zeros(n, f)
    r = np.array(b, f)
    z = self.vcycle(0, r)
    if self.cg_alias and len(self.levels) > 1:
      r = self._vres.copy()
    p = z.copy()
    rz = float(np.dot(r.astype(np.float64), z.astype(np.float64)))
    rr0 = float(np.dot(np.asarray(b, np.float64), np.asarray(b, np.float64)))
    tol2 = max(self.tol_cg ** 2, self.rel_tol_cg ** 2 * rr0)
    it = 0
    for k in range(self.maxiter_cg):
      ap = (A @ p).astype(f)
      pap = float(np.dot(p.astype(np.float64), ap.astype(np.float64)))
      if abs(pap) < 1e-30:
        break
      alpha = rz / pap
      x = (x + f(alpha) * p).astype(f)
      r = (r + f(-alpha) * ap).astype(f)
      rr = float(np.dot(r.astype(np.float64), r.astype(np.float64)))
      if rr < tol2:
        it = k + 1
        break
      z = self.vcycle(0, r)
      if self.cg_alias and len(self.levels) > 1:
        r = self._vres.copy()
      rz_new = float(np.dot(r.astype(np.float64), z.astype(np.float64)))
      if abs(rz) < 1e-30:
        it = k + 1
        break
      beta = rz_new / rz
      p = (z + f(beta) * p).astype(f)
      rz = rz_new
      it = k + 1
    return x, it

  def residual(self):
    f = self.dtype
    b = (-(self.C + self.alpha * self.lam)).astype(f)
    return b, float(np.sqrt(np.dot(b.astype(np.float64), b.astype(np.float64))))

  # _scatter_dlam_gpu (cons/mgpbd_gpu.py:330-343), serial tet order
  def scatter(self, dlam):
    f = self.dtype
    self.lam = (self.lam + dlam).astype(f)
    t = self.t_i.reshape(-1, 4)
    contrib = (self.invm[t] * dlam[:, None])[:, :, None] * self.gradC
    dpos = np.zeros((self.nv, 3), f)
    np.add.at(dpos, t.reshape(-1), contrib.reshape(-1, 3).astype(f))
    self.dpos = dpos

  def dual_norm_at(self, pos):
    f = self.dtype
    c = constraint_values(pos, self.t_i, self.dm_inv, f, self.ctype, self.rest_vol)
    r = (-(c + self.alpha * self.lam)).astype(np.float64)
    return float(np.sqrt(np.dot(r, r)))

  # cons/mgpbd_gpu.py:379-391
  def line_search(self, beta=0.5, max_steps=10):
    f = self.dtype
    current = self.dual_norm_at(self.x)
    omega = 1.0
    for _ in range(max_steps):
      trial = (self.x + f(omega) * self.dpos).astype(f)
      if self.dual_norm_at(trial) < current:
        return omega
      omega *= beta
    return omega

  def apply(self, omega):
    f = self.dtype
    m = self.invm > 0
    self.x[m] = (self.x + f(omega) * self.dpos).astype(f)[m]

  # cons/mgpbd_gpu.py:397-446
  def solve(self, frame=0):
    f = self.dtype
    self.lam = np.zeros(self.nt, f)
    r0 = 0.0
    self.log = []
    for ite in range(self.maxiter):
      self.C, self.gradC = constraints(self.x, self.t_i, self.dm_inv, f, self.ctype,
                                       self.rest_vol)
      b, r = self.residual()
      if ite == 0:
        r0 = r
      if r < self.atol or (r0 > 1e-12 and r < self.rtol * r0):
        self.log.append((ite, r, 0, 1.0))
        break
      if self.linear == 'exact':
        from .exact_solve import ExactDualSolve
        ex = ExactDualSolve(self.t_i, self.gradC, self.invm, self.alpha)
        dlam, rel = ex.solve(b, self.exact_tol)
        self.exact_log.append((ite, rel, list(ex.iters)))
        it = 0
      elif self.linear == 'cheb':
        from .exact_solve import chebyshev_pcg, constraint_jacobian
        J = constraint_jacobian(self.t_i, self.gradC, self.nv)
        Jt = J.T.tocsr()
        w3 = np.repeat(np.asarray(self.invm, np.float64), 3)
        al = np.asarray(self.alpha, np.float64)
        x0 = self.dlam_prev if (self.warm_substep and ite == 0) else None
        dlam, it = chebyshev_pcg(lambda v: al * v + J @ (w3 * (Jt @ v)), b,
                                 rel_tol=self.rel_tol_cg, tol_abs=self.tol_cg,
                                 maxiter=self.maxiter_cg, x0=x0)
        if self.warm_substep and ite == 0:
          self.dlam_prev = dlam.copy()
      else:
        self.fill_matrices()
        dlam, it = self.pcg(b)
      self.scatter(dlam)
      omega = self.line_search() if self.use_line_search else 1.0
      self.apply(omega)
      self.log.append((ite, r, it, omega))


# ---------------------------------------------------------------------------
# Adaptive zones (cons/adaptive_zone.py:40-85), float32 like the reference.

def zone_proximity(x, t_i, center, radius):
  """cons/adaptive_zone.py:40-55: 1 iff a vertex is strictly within radius."""
  t = np.asarray(t_i).reshape(-1, 4)
  p = np.asarray(x, np.float32)[t]                     # (nt, 4, 3)
  d = p - np.asarray(center, np.float32)
  d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
  r2 = np.float32(radius) * np.float32(radius)
  return (d2 < r2).any(axis=1).astype(np.int32)


def zone_strain(x, x_old, t_i, threshold, dt):
  """cons/adaptive_zone.py:57-72: 1 iff the fastest vertex moved faster
  than threshold (speed = |x - x_old| / dt)."""
  t = np.asarray(t_i).reshape(-1, 4)
  d = np.asarray(x, np.float32)[t] - np.asarray(x_old, np.float32)[t]
  n2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
  speed = np.sqrt(n2) / np.float32(dt)
  vmax = np.maximum(speed.max(axis=1), np.float32(0.0))
  return (vmax > np.float32(threshold)).astype(np.int32)


def zone_expand(active, adj, n_rings):
  """cons/adaptive_zone.py:74-85 with adj from face_adjacency_sets."""
  active = np.asarray(active, np.int32).copy()
  for _ in range(n_rings):
    new = active.copy()
    for t in range(len(active)):
      if active[t] == 1:
        for nb in adj[t]:
          new[nb] = 1
    active = new
  return active
