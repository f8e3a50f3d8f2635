"""Length + volume constraint discretisation (one length constraint per
unique tet edge, one volume constraint det F - 1 per tet): the system
builder and its hierarchy (CPU), the oracle's gradients against finite
differences (CPU), and the CUDA step against the float64 oracle on the same
constraints (GPU, per stage and per substep, plain V-cycle and FAST paths).

These blocks have no reference counterpart in the MGPBD step (the reference
uses one ARAP constraint per tet); their definitions follow cons/length.py
(C = |x_a - x_b| - L0) and the hydrostatic constraint of cons/deform3d.py
(C = det F - 1), and the oracle is this project's float64 restatement.
Tolerances as in test_gpu_parity: per-stage 1e-4 relative (C 1e-5),
positions 1e-5 relative.
"""

import numpy as np
import pytest

from controllable_pbd_3d_gb300 import _native as N
from controllable_pbd_3d_gb300 import meshgen
from controllable_pbd_3d_gb300.edge_volume import edge_volume_hierarchy, edge_volume_system
from oracle import mgpbd_oracle as MO


def body(n=5, jitter=0.03, seed=2):
  xr, t = meshgen.hex_grid_tets(n, n, n, h=1.0 / n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, h=1.0 / n, jitter=jitter, seed=seed)
  invm = np.ones(len(xr), np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  return xr, x0, t, invm


def test_system_builder():
  _, _, t, _ = body(6)
  q = t.reshape(-1, 4)
  c, types, edges, owner = edge_volume_system(t)
  nt = len(q)
  assert len(types) == nt + len(edges) and len(c) == 4 * len(types)
  assert (types[:nt] == N.MGPBD_CONS_VOLUME).all() and (types[nt:] == N.MGPBD_CONS_LENGTH).all()
  cc = c.reshape(-1, 4)
  assert np.array_equal(cc[:nt], q)
  assert np.array_equal(cc[nt:, :2], edges) and np.array_equal(cc[nt:, 2:], edges)
  # every tet edge exactly once, sorted, owned by the first tet that has it
  allk = set()
  for ti, tt in enumerate(q):
    for a in range(4):
      for b in range(a + 1, 4):
        allk.add(tuple(sorted((int(tt[a]), int(tt[b])))))
  assert len(allk) == len(edges) and (edges[:, 0] < edges[:, 1]).all()
  assert [tuple(e) for e in edges] == sorted(allk)
  assert edge_volume_hierarchy(meshgen.hex_grid_tets(4, 4, 4)[1]) is None  # 320 tets: one level
  for (a, b), o in zip(edges[:50], owner[:50]):
    has = [i for i, tt in enumerate(q) if a in tt and b in tt]
    assert o == min(has)
  agg = edge_volume_hierarchy(t)
  from controllable_pbd_3d_gb300.tet_aggregation import build_tet_hierarchy
  Ps, sizes = build_tet_hierarchy(t, None, nt)
  assert np.array_equal(agg[:nt], Ps[0].indices)
  assert np.array_equal(agg[nt:], Ps[0].indices[owner])
  assert set(np.unique(agg)) == set(range(sizes[1]))


def test_oracle_gradients_match_finite_differences():
  xr, x0, t, _ = body(3, 0.08, 5)
  c, types, _, _ = edge_volume_system(t)
  dm, rest, _ = MO.rest_shape(xr, c, 1.0, 1.0, np.float64, 1e-6, types)
  C, g = MO.constraints(x0, c, dm, np.float64, types, rest)
  x = x0.astype(np.float64)
  cc = c.reshape(-1, 4)
  rng = np.random.default_rng(0)
  h = 1e-7
  for k in rng.choice(len(types), 40, replace=False):
    # a vertex listed twice (length constraints: a, b, a, b) gets the sum of
    # its slots' gradients (the repeated slots carry zero)
    for v in sorted(set(int(q) for q in cc[k])):
      for d in range(3):
        xp = x.copy()
        xp[v, d] += h
        xm = x.copy()
        xm[v, d] -= h
        one = cc[k:k + 1].reshape(-1)
        fd = (MO.constraint_values(xp, one, dm[k:k + 1], np.float64, types[k:k + 1],
                                   rest[k:k + 1])[0] -
              MO.constraint_values(xm, one, dm[k:k + 1], np.float64, types[k:k + 1],
                                   rest[k:k + 1])[0]) / (2 * h)
        want = sum(g[k, s2, d] for s2 in range(4) if cc[k, s2] == v)
        assert abs(fd - want) <= 1e-5 * max(1.0, abs(want)), (k, v, d, fd, want)
    if types[k] == N.MGPBD_CONS_LENGTH:
      assert np.all(g[k, 2:] == 0)
  # rest state: zero constraint values
  C0, _ = MO.constraints(xr, c, dm, np.float64, types, rest)
  assert np.abs(C0).max() < 1e-6


def test_oracle_step_converges():
  xr, x0, t, invm = body(5)
  c, types, _, _ = edge_volume_system(t)
  agg = edge_volume_hierarchy(t)
  o = MO.MGPBDOracle(x0, xr, invm, c, [0, -9.8, 0], 1 / 300, dtype=np.float64, compliance=1e-6,
                     ctype=types, hierarchy=([agg], [len(types), int(agg.max()) + 1]),
                     kinematic_pins=True, maxiter=5, maxiter_cg=2000, rel_tol_cg=1e-8,
                     tol_cg=1e-14, smoother='safe')
  o.init()
  o.step(0)
  assert np.isfinite(o.x).all()
  b, r = o.residual()
  assert r < o.log[0][1]


def gpu_solver(torch, xr, x0, t, invm, **kw):
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  x = torch.tensor(x0, device='cuda')
  s = MGPBDSolverGPU(x, torch.tensor(xr, device='cuda'), torch.tensor(invm, device='cuda'),
                     torch.tensor(t, device='cuda'), None, [0.0, -9.8, 0.0], 1.0 / 300,
                     constraints='edge_volume', compliance=1e-6, kinematic_pins=True, **kw)
  s.init()
  return s, x


def oracle(xr, x0, t, invm, **kw):
  c, types, _, _ = edge_volume_system(t)
  agg = edge_volume_hierarchy(t)
  o = MO.MGPBDOracle(x0, xr, invm, c, [0, -9.8, 0], 1 / 300, compliance=1e-6, ctype=types,
                     hierarchy=([agg], [len(types), int(agg.max()) + 1]), kinematic_pins=True,
                     **kw)
  o.init()
  return o


@pytest.mark.gpu
def test_gpu_stages_match_oracle(cuda):
  torch = cuda
  xr, x0, t, invm = body(6)
  s, x = gpu_solver(torch, xr, x0, t, invm)
  o = oracle(xr, x0, t, invm, dtype=np.float32)
  assert np.allclose(s.rest_vol.cpu().numpy(), o.rest_vol, rtol=1e-5)
  assert np.allclose(s.alpha_tilde.cpu().numpy(), o.alpha, rtol=1e-6)
  s._compute_C_and_gradC()
  C = s.constraints.cpu().numpy()
  g = s.gradC.cpu().numpy()
  Co, go = MO.constraints(x0, o.t_i, o.dm_inv, np.float32, o.ctype, o.rest_vol)
  assert np.abs(C - Co).max() <= 1e-5 * max(np.abs(Co).max(), 1e-3)
  assert np.abs(g - go).max() <= 1e-4 * np.abs(go).max()
  s._residual_norm_gpu()
  s._fill_A_and_update_gpu()
  A = s._gpu_solver._gpu_As[0].data.cpu().numpy()
  Ao = MO.fill_A(o.levels[0].indptr, o.levels[0].indices, o.t_i, o.invm, go, o.alpha,
                 np.float32)
  assert np.abs(A - Ao).max() <= 1e-4 * np.abs(Ao).max()


VARIANTS = {
    'vcycle': dict(smoother='safe'),
    'fast-primal': dict(mode='fast', precond='cheb', cheb_lo=1e-3, primal=True, primal_tol=1e-2),
    # the persistent kernels reading the operator from L2, with the length
    # constraints in compact two-vertex form (the path of large meshes)
    'fast-primal-l2': dict(mode='fast', precond='cheb', cheb_lo=1e-3, primal=True,
                           primal_tol=1e-2, persistent=2),
    'fast-dual-l2': dict(mode='fast', precond='cheb', cheb_lo=1e-3, primal=False, persistent=2),
    # the Chebyshev polynomial on A itself (no Jacobi scaling): staged, from
    # L2, with the primal warm start, and as per-phase kernels
    'fast-unscaled': dict(mode='fast', precond='cheb', cheb_lo=1e-3, cheb_scale='none',
                          primal=False),
    'fast-unscaled-l2': dict(mode='fast', precond='cheb', cheb_lo=1e-3, cheb_scale='none',
                             primal=False, persistent=2),
    'fast-unscaled-primal': dict(mode='fast', precond='cheb', cheb_lo=1e-3, cheb_scale='none',
                                 primal=True, primal_tol=1e-2),
    'fast-unscaled-kernels': dict(mode='fast', precond='cheb', cheb_lo=1e-3, cheb_scale='none',
                                  primal=False, persistent=0),
}


@pytest.mark.gpu
@pytest.mark.parametrize('variant', list(VARIANTS))
def test_gpu_substeps_match_float64_oracle(cuda, variant):
  torch = cuda
  xr, x0, t, invm = body(6)
  kw = dict(damp=0.993, maxiter=5, rtol=1e-6, atol=1e-9, maxiter_cg=4000, tol_cg=1e-12,
            rel_tol_cg=1e-7)
  o = oracle(xr, x0, t, invm, dtype=np.float64, smoother='safe', **kw)
  extra = VARIANTS[variant]
  s, x = gpu_solver(torch, xr, x0, t, invm, **kw, **extra)
  for k in range(2):
    o.step(k)
    s.step(k)
  err = float(np.abs(x.cpu().numpy() - o.x).max())
  assert err <= 1e-5 * float(np.abs(o.x).max()), err
  assert s.stats()['newton_iters'] >= 1
  if variant.endswith('-l2'):
    assert s.stats()['cg_path'] in ('persistent', 'primal')  # unstaged


@pytest.mark.gpu
def test_gpu_rejects_a_bad_length_constraint(cuda):
  torch = cuda
  from controllable_pbd_3d_gb300.mgpbd_gpu import MGPBDSolverGPU
  from controllable_pbd_3d_gb300._native import MGPBDError
  xr, x0, t, invm = body(3)
  c, types, _, _ = edge_volume_system(t)
  c = c.copy()
  c[4 * (len(types) - 1) + 2] = c[4 * (len(types) - 1) + 1]  # (a, b, b, b)
  s = MGPBDSolverGPU(torch.tensor(x0, device='cuda'), torch.tensor(xr, device='cuda'),
                     torch.tensor(invm, device='cuda'), torch.tensor(c, device='cuda'), None,
                     [0.0, -9.8, 0.0], 1.0 / 300, compliance=1e-6)
  import ctypes as C
  N.check(s._lib.mgpbd_set_constraint_types(s._h, types.ctypes.data), 'types')
  with pytest.raises(MGPBDError):
    s.init()


def test_oracle_length_constraint_replays_the_reference_sweep():
  """One Gauss-Seidel sweep of the reference's own length constraints
  (cons/length.py, `tests/golden/length.npz` from `make_golden.py --only
  length`) replayed with the oracle's length C and slot gradients (slots a,
  b, a, b): same positions and multipliers to float32 rounding."""
  from conftest import golden
  z = golden('length.npz')
  x = z['x0'].astype(np.float64)
  edges, rest, invm = z['edges'], z['rest'], z['invm'].astype(np.float64)
  alpha = float(z['compliance']) / float(z['dt']) ** 2
  lam = np.zeros(len(edges))
  dm0 = np.zeros((1, 3, 3))
  for k, (a, b) in enumerate(edges):
    t4 = np.array([a, b, a, b], np.int32)
    c, g = MO.constraints(x, t4, dm0, np.float64, ctype=[MO.CONS_LENGTH], rest=rest[k:k + 1])
    g = g.reshape(4, 3)
    assert np.allclose(g[2:], 0) and np.allclose(g[0], -g[1])
    d = -(c[0] + alpha * lam[k]) / (invm[a] * (g[0] @ g[0]) + invm[b] * (g[1] @ g[1]) + alpha)
    lam[k] += d
    x[a] += invm[a] * d * g[0]
    x[b] += invm[b] * d * g[1]
  assert np.abs(x - z['x1']).max() <= 2e-6
  assert np.allclose(lam, z['lam'], rtol=1e-4, atol=1e-7)
  assert np.abs(z['lam']).max() > 1e-3  # the sweep did move the body


def test_oracle_volume_constraint_is_the_local_hydrostatic_constraint():
  """C = det F - 1 and its four slot gradients from the MGPBD oracle equal
  the hydrostatic constraint of the local XPBD oracle (cons/deform3d.py:
  81-83), whose substeps are pinned to the reference's own Deform3D
  (`test_local.py`)."""
  from oracle import local_oracle as LO
  xr, t = meshgen.hex_grid_tets(3, 3, 2)
  x, _ = meshgen.hex_grid_tets(3, 3, 2, jitter=0.2, seed=8)
  x = x.astype(np.float64)
  nt = len(t) // 4
  dm_inv, _, _ = MO.rest_shape(xr, t, 1e5, 1 / 300, np.float64)
  c, g = MO.constraints(x, t, dm_inv, np.float64, ctype=np.full(nt, MO.CONS_VOLUME))
  B, _ = LO.rest_shape(xr.astype(np.float64), t.reshape(-1, 4))
  q = t.reshape(-1, 4).astype(np.int64)
  F = LO._deformation(x, q, B)
  gH3 = LO._cof(F) @ np.transpose(B, (0, 2, 1))
  gH = np.concatenate([np.transpose(gH3, (0, 2, 1)), -gH3.sum(axis=2)[:, None, :]], axis=1)
  assert np.allclose(c, np.linalg.det(F) - 1.0, rtol=0, atol=1e-12)
  assert np.allclose(g.reshape(nt, 4, 3), gH, rtol=1e-10, atol=1e-10)


def test_cpp_structure_matches_oracle_on_the_length_volume_system():
  """Level-0 pattern (constraints sharing a vertex, itself last) and the
  Galerkin pattern and contribution map of the length + volume system,
  whose length constraints repeat their vertices (a, b, a, b): the C++
  builders equal the oracle bit for bit."""
  from controllable_pbd_3d_gb300 import tet_aggregation as ta
  xr, t = meshgen.hex_grid_tets(6, 5, 4, jitter=0.05, seed=9)
  c, types, _, _ = edge_volume_system(t)
  nc = len(types)
  ip, ix = ta.sparsity_pattern(c, nc)
  ip2, ix2 = MO.sparsity_pattern(c, nc)
  np.testing.assert_array_equal(ip, ip2)
  np.testing.assert_array_equal(ix, ix2)
  rows = np.repeat(np.arange(nc), np.diff(ip))
  assert (ix[ip[1:] - 1] == np.arange(nc)).all()  # the constraint itself last
  assert len(np.unique(rows * nc + ix)) == len(ix)  # no duplicate columns
  agg = edge_volume_hierarchy(t)
  n1 = int(agg.max()) + 1
  rng = np.random.default_rng(3)
  data = rng.standard_normal(len(ix)).astype(np.float32)
  data[rng.random(len(ix)) < 0.2] = 0.0
  ci, cx, cidx, coff = ta.galerkin_structure(ip, ix, data, agg, n1)
  ci2, cx2, cidx2, coff2, _ = MO.galerkin(ip2, ix2, data, agg, n1)
  np.testing.assert_array_equal(ci, ci2)
  np.testing.assert_array_equal(cx, cx2)
  np.testing.assert_array_equal(cidx, cidx2)
  np.testing.assert_array_equal(coff, coff2)


def test_vertex_incidence_leaves_out_repeated_slots():
  """The operator's vertex incidence (host builder of the library) against a
  numpy restatement: 4 * t + l per slot naming the vertex, ascending t, the
  repeated slots of length constraints (a, b, a, b) left out; bad ids are
  rejected."""
  from controllable_pbd_3d_gb300 import tet_aggregation as ta
  xr, t = meshgen.hex_grid_tets(4, 3, 3)
  c, types, _, _ = edge_volume_system(t)
  nc, nv = len(types), len(xr)
  ptr, ent = ta.vertex_incidence(c, nc, nv)
  q = c.reshape(-1, 4)
  keep = np.ones_like(q, bool)
  for l in range(1, 4):
    keep[:, l] = ~(q[:, :l] == q[:, l:l + 1]).any(axis=1)
  slot = (4 * np.arange(nc)[:, None] + np.arange(4)[None, :])[keep]
  vert = q[keep]
  order = np.lexsort((slot, vert))
  assert np.array_equal(ent, slot[order])
  assert np.array_equal(ptr, np.concatenate([[0], np.cumsum(np.bincount(vert, minlength=nv))]))
  assert len(ent) == 4 * int((types == MO.CONS_VOLUME).sum()) + 2 * int((types == MO.CONS_LENGTH).sum())
  bad = c.copy()
  bad[5] = nv
  with pytest.raises(Exception):
    ta.vertex_incidence(bad, nc, nv)
