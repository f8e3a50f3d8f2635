"""Comparison solvers of the convergence experiments: greedy colourings
(utils/graph_coloring.py), local XPBD `Deform3D` (cons/deform3d.py) and
`VBDSolver` (cons/vbd.py).

CPU: the library's host colourings against the reference's own colourings
(golden, bit-exact) and the oracle restatement (random graphs); the float64
oracle against the reference's substeps (golden).  GPU: the CUDA solvers
against the same golden substeps and against the oracle on larger meshes,
colour kernels run twice for determinism.
"""


import numpy as np
import pytest

from conftest import golden
from controllable_pbd_3d_gb300 import graph_coloring as gcol
from controllable_pbd_3d_gb300 import meshgen
from controllable_pbd_3d_gb300._native import MGPBDError
from oracle import local_oracle as LO

COLOR_CASES = ('box5x4x5', 'cube6', 'box12x3x7', 'simple_sphere', 'spot', 'cube_tet')
XPBD_CASES = ('xpbd_gs_box', 'xpbd_color_box', 'xpbd_gs_sphere', 'xpbd_default_disjoint')
VBD_CASES = ('vbd_serial_box', 'vbd_color_box', 'vbd_color_cheb_box', 'vbd_serial_sphere')


def case(name):
  z = golden('local.npz')
  p = name + '/'
  return {k[len(p):]: z[k] for k in z.files if k.startswith(p)}


def kwargs(d):
  out = {}
  for k, v in d.items():
    if k.startswith('kw_'):
      out[k[3:]] = str(v) if v.dtype.kind == 'U' else v.item()
  return out


# ---------------------------------------------------------------------------
# colourings (host)


@pytest.mark.parametrize('name', COLOR_CASES)
def test_colorings_match_reference(name):
  d = case('color/' + name)
  t, nv = d['t_i'], int(d['nv'])
  nt = len(t) // 4
  ce = gcol.color_elements(t, nt, 4, nv)
  assert np.array_equal(ce.ordered_indices, d['elem_ordered'])
  assert ce.color_offsets == d['elem_offsets'].tolist()
  assert ce.num_colors == len(d['elem_offsets']) - 1
  cv = gcol.color_vertices(t, nt, 4, nv)
  assert np.array_equal(cv.ordered_indices, d['vert_ordered'])
  assert cv.color_offsets == d['vert_offsets'].tolist()


def test_coloring_is_proper():
  _, t = meshgen.hex_grid_tets(5, 4, 3)
  nv, nt = int(t.max()) + 1, len(t) // 4
  q = t.reshape(-1, 4)
  ce = gcol.color_elements(t, nt, 4, nv)
  for c in range(ce.num_colors):
    tets = ce.ordered_indices[ce.color_offsets[c]:ce.color_offsets[c + 1]]
    vs = q[tets].reshape(-1)
    assert len(np.unique(vs)) == len(vs)  # no shared vertex inside a colour
  cv = gcol.color_vertices(t, nt, 4, nv)
  col = np.empty(nv, np.int64)
  for c in range(cv.num_colors):
    col[cv.ordered_indices[cv.color_offsets[c]:cv.color_offsets[c + 1]]] = c
  for row in q:
    assert len(np.unique(col[row])) == 4  # no two vertices of a tet share a colour


@pytest.mark.parametrize('seed', range(6))
def test_greedy_matches_oracle_on_random_graphs(seed):
  rng = np.random.default_rng(seed)
  n = int(rng.integers(0, 60))
  adj = [set() for _ in range(n)]
  for _ in range(int(rng.integers(0, 4 * n + 1))):
    i, j = (int(v) for v in rng.integers(0, max(n, 1), 2))
    if n:
      adj[i].add(j)  # self loops and one-sided edges included
      adj[j].add(i)
  r = gcol.greedy_coloring(adj, n)
  o_ord, o_off, o_n = LO.greedy(adj, n)
  assert np.array_equal(r.ordered_indices, o_ord)
  assert r.color_offsets == o_off.tolist()
  assert r.num_colors == o_n


@pytest.mark.parametrize('k', [2, 3, 4])
def test_element_and_vertex_coloring_match_oracle(k):
  rng = np.random.default_rng(k)
  nv, ne = 40, 70
  e = rng.integers(0, nv, ne * k).astype(np.int32)  # repeated vertices allowed
  for fn, ofn, n in ((gcol.color_elements, LO.color_elements, ne),
                     (gcol.color_vertices, LO.color_vertices, nv)):
    r = fn(e, ne, k, nv)
    o_ord, o_off, _ = ofn(e.tolist(), ne, k, nv)
    assert np.array_equal(r.ordered_indices, o_ord)
    assert r.color_offsets == o_off.tolist()
    assert len(r.ordered_indices) == n
  ce = gcol.color_edges(e[:2 * ne], ne, nv)
  o_ord, _, _ = LO.color_elements(e[:2 * ne].tolist(), ne, 2, nv)
  assert np.array_equal(ce.ordered_indices, o_ord)


def test_build_adjacency_matches_oracle():
  _, t = meshgen.hex_grid_tets(3, 2, 2)
  nv, nt = int(t.max()) + 1, len(t) // 4
  assert gcol.build_element_adjacency(t, nt, 4, nv) == LO.element_adjacency(t.tolist(), nt, 4, nv)
  assert gcol.build_vertex_adjacency(t, nt, 4, nv) == LO.vertex_adjacency(t.tolist(), nt, 4, nv)


def test_coloring_edge_cases():
  r = gcol.color_elements(np.zeros(0, np.int32), 0, 4, 0)
  assert r.num_colors == 0 and r.color_offsets == [0] and len(r.ordered_indices) == 0
  r = gcol.greedy_coloring([], 0)
  assert r.num_colors == 0
  with pytest.raises(MGPBDError):
    gcol.color_vertices(np.array([0, 1, 2, 9], np.int32), 1, 4, 4)
  with pytest.raises(MGPBDError):
    gcol.color_elements(np.array([0, -1], np.int32), 1, 2, 4)
  with pytest.raises(ValueError):
    gcol.color_elements(np.array([0, 1], np.int32), 1, 2, 2, algorithm='dsatur')


# ---------------------------------------------------------------------------
# the oracle against the reference's substeps


def run_oracle_xpbd(d, coloring=None):
  x = d['x0'].astype(np.float64)
  fw = LO.Framework(x, d['gravity'], float(d['dt']), float(d['damp']))
  kw = kwargs(d)
  c = LO.Deform3D(x, d['x_ref'], d['invm'], d['t_i'], d['t_m'], float(d['dt']),
                  kw['hydro_alpha'], kw['devia_alpha'], kw['method'], coloring=coloring)
  fw.cons.append(c)
  traj = []
  for _ in range(int(d['substeps'])):
    fw.step(int(d['passes']))
    traj.append(x.copy())
  return np.stack(traj), c, fw


def run_oracle_vbd(d):
  x = d['x0'].astype(np.float64)
  s = LO.VBD(x, d['x_ref'], d['invm'], d['t_i'], d['gravity'], float(d['dt']),
             damp=float(d['damp']), **kwargs(d))
  traj = []
  for _ in range(int(d['substeps'])):
    s.step()
    traj.append(x.copy())
  return np.stack(traj), s


@pytest.mark.parametrize('name', XPBD_CASES)
def test_oracle_xpbd_matches_reference(name):
  d = case(name)
  traj, c, fw = run_oracle_xpbd(d)
  assert np.abs(traj - d['x_traj']).max() < 5e-6
  assert np.abs(fw.v - d['v_final']).max() < 5e-6 / float(d['dt'])
  scale = np.abs(d['devia_lambda']).max()
  assert np.abs(c.ld - d['devia_lambda']).max() < 1e-3 * scale


@pytest.mark.parametrize('name', VBD_CASES)
def test_oracle_vbd_matches_reference(name):
  d = case(name)
  traj, s = run_oracle_vbd(d)
  assert np.abs(traj - d['x_traj']).max() < 5e-6
  assert np.allclose(s.Dm_inv, d['dm_inv'], rtol=1e-5, atol=1e-5 * np.abs(d['dm_inv']).max())
  assert np.array_equal(s.adj_tet, d['adj_tets']) and np.array_equal(s.adj_loc, d['adj_local'])
  assert np.allclose([s.mu, s.lam], d['mu_lam'], rtol=1e-12)


# ---------------------------------------------------------------------------
# the CUDA solvers (through libmgpbd.so)


def gpu_xpbd(torch, d, method=None):
  from controllable_pbd_3d_gb300 import Deform3D, PbdFramework
  x = torch.tensor(d['x0'], device='cuda')
  kw = kwargs(d)
  if method is not None:
    kw['method'] = method
  c = Deform3D(x, d['x_ref'], d['invm'], d['t_i'], d['t_m'], float(d['dt']), **kw)
  fw = PbdFramework(x, d['gravity'].tolist(), float(d['dt']), float(d['damp']))
  fw.add_cons(c)
  fw.init_rest_status()
  traj = []
  for _ in range(int(d['substeps'])):
    fw.step(int(d['passes']))
    traj.append(x.cpu().numpy())
  c.synchronize()  # raises if a colour kernel's grid barrier gave up
  return np.stack(traj), c, fw


def gpu_vbd(torch, d, **over):
  from controllable_pbd_3d_gb300 import VBDSolver
  x = torch.tensor(d['x0'], device='cuda')
  kw = kwargs(d)
  kw.update(over)
  s = VBDSolver(x, d['x_ref'], d['invm'], d['t_i'], d['t_m'], d['gravity'].tolist(),
                float(d['dt']), damp=float(d['damp']), **kw)
  s.init()
  traj = []
  for k in range(int(d['substeps'])):
    s.step(k)
    traj.append(x.cpu().numpy())
  s.synchronize()
  return np.stack(traj), s


@pytest.mark.gpu
@pytest.mark.parametrize('name', XPBD_CASES)
def test_gpu_xpbd_matches_reference(cuda, name):
  d = case(name)
  traj, c, fw = gpu_xpbd(cuda, d)
  # float32 on both sides, different contraction and summation order
  assert np.abs(traj - d['x_traj']).max() < 2e-5
  assert np.abs(fw.v_v.cpu().numpy() - d['v_final']).max() < 2e-5 / float(d['dt'])
  scale = np.abs(d['devia_lambda']).max()
  assert np.abs(c.devia_lambda.cpu().numpy() - d['devia_lambda']).max() < 5e-3 * scale


@pytest.mark.gpu
@pytest.mark.parametrize('name', VBD_CASES)
def test_gpu_vbd_matches_reference(cuda, name):
  d = case(name)
  traj, s = gpu_vbd(cuda, d)
  assert np.abs(traj - d['x_traj']).max() < 2e-5
  assert np.allclose(s.Dm_inv.cpu().numpy(), d['dm_inv'], rtol=1e-4,
                     atol=1e-5 * np.abs(d['dm_inv']).max())
  assert np.allclose(s.rest_vol.cpu().numpy(), d['rest_vol'], rtol=1e-5)
  assert np.allclose([s.mu, s.lam], d['mu_lam'], rtol=1e-6)


def grid_body(n, jitter, seed):
  xr, t = meshgen.hex_grid_tets(n, n, n)
  x0, _ = meshgen.hex_grid_tets(n, n, n, jitter=jitter, seed=seed)
  vm = np.zeros(len(xr))
  q = t.reshape(-1, 4)
  _, vol = LO.rest_shape(xr, t)
  np.add.at(vm, q.reshape(-1), np.repeat(vol / 4.0, 4))
  invm = (1.0 / vm).astype(np.float32)
  invm[meshgen.grid_face_vertices(n, n, n, axis=1, side='max')] = 0.0
  return {'x_ref': xr.astype(np.float32), 'x0': x0.astype(np.float32), 't_i': t.astype(np.int32),
          'invm': invm, 't_m': vol.astype(np.float32),
          'gravity': np.array([0.0, -9.8, 0.0], np.float32), 'dt': np.array(1.0 / 300.0),
          'damp': np.array(0.993), 'substeps': np.array(3), 'passes': np.array(10)}


@pytest.mark.gpu
def test_gpu_xpbd_colour_matches_oracle_12cube(cuda):
  d = grid_body(12, 0.05, 4)
  d.update(kw_hydro_alpha=np.array(1e-5), kw_devia_alpha=np.array(1e-4),
           kw_method=np.array('graph_coloring'))
  traj, c, _ = gpu_xpbd(cuda, d)
  otraj, oc, _ = run_oracle_xpbd(d)
  assert np.isfinite(traj).all()
  assert np.abs(traj - otraj).max() < 5e-5
  assert c.num_colors == len(oc.offsets) - 1


@pytest.mark.gpu
def test_gpu_vbd_colour_matches_oracle_12cube(cuda):
  d = grid_body(12, 0.05, 4)
  d.update(kw_youngs_modulus=np.array(1e4), kw_poissons_ratio=np.array(0.3),
           kw_n_iterations=np.array(10), kw_rho=np.array(0.5), kw_damping=np.array(0.02),
           kw_method=np.array('color'))
  traj, s = gpu_vbd(cuda, d)
  otraj, os_ = run_oracle_vbd(d)
  assert np.isfinite(traj).all()
  assert np.abs(traj - otraj).max() < 5e-5
  assert np.allclose(s._omegas, os_.omegas, rtol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize('solver', ['xpbd', 'vbd'])
def test_gpu_colour_kernels_are_deterministic(cuda, solver):
  d = grid_body(10, 0.05, 9)
  if solver == 'xpbd':
    d.update(kw_hydro_alpha=np.array(0.0), kw_devia_alpha=np.array(1e-4),
             kw_method=np.array('graph_coloring'))
    a, _, _ = gpu_xpbd(cuda, d)
    b, _, _ = gpu_xpbd(cuda, d)
  else:
    d.update(kw_youngs_modulus=np.array(1e4), kw_poissons_ratio=np.array(0.3),
             kw_n_iterations=np.array(6), kw_method=np.array('color'))
    a, _ = gpu_vbd(cuda, d)
    b, _ = gpu_vbd(cuda, d)
  assert np.array_equal(a, b)


def devia_violation(x, xr, t):
  B, _ = LO.rest_shape(xr, t)
  F = LO._deformation(np.asarray(x, np.float64), t.reshape(-1, 4).astype(np.int64), B)
  return np.abs(np.einsum('mij,mij->m', F, F) - 3.0).mean()


@pytest.mark.gpu
def test_gpu_xpbd_default_method_relaxes_a_shared_mesh(cuda):
  """The parallel method applies every tet's correction at once (a vertex
  of this grid takes ~20 corrections per pass, with racy reads, like the
  reference's parallel loop), i.e. a Jacobi iteration: with stiff
  constraints (hydro_alpha = 0 makes det F = 1 a hard constraint) it
  overshoots and diverges, as Jacobi does.  In the compliant regime (alpha~
  ~ 12x the deviatoric constraint's stiffness) it must stay finite, reduce
  the deviatoric violation and land near the Gauss-Seidel result (a float64
  Jacobi pass lands within 2 % of the displacement)."""
  d = grid_body(10, 0.05, 2)
  d.update(gravity=np.zeros(3, np.float32), kw_hydro_alpha=np.array(0.1),
           kw_devia_alpha=np.array(0.1), kw_method=np.array('default'), substeps=np.array(1))
  traj, c, _ = gpu_xpbd(cuda, d)
  gs, _, _ = gpu_xpbd(cuda, d, method='gauss_seidel')
  assert np.isfinite(traj).all()
  assert devia_violation(traj[-1], d['x_ref'], d['t_i']) < devia_violation(
      d['x0'], d['x_ref'], d['t_i'])
  assert np.abs(c.devia_lambda.cpu().numpy()).max() > 0.0
  moved = np.abs(gs[-1] - d['x0']).max()
  assert moved > 0.0
  assert np.abs(traj[-1] - gs[-1]).max() < 0.1 * moved


@pytest.mark.gpu
def test_gpu_local_solvers_40cube_properties(cuda):
  """At the benchmark size (40^3 cube, 320k tets): one colour pass of XPBD
  and two VBD iterations stay finite, pinned vertices stay put, and the XPBD
  pass equals the float64 oracle's colour pass to float32 accuracy (the
  oracle follows the library's tet colouring, which the reference's own
  colourings pin bit for bit on smaller meshes)."""
  d = grid_body(40, 0.01, 0)
  d.update(kw_hydro_alpha=np.array(1e-5), kw_devia_alpha=np.array(1e-4),
           kw_method=np.array('graph_coloring'), substeps=np.array(1), passes=np.array(1))
  traj, c, _ = gpu_xpbd(cuda, d)
  col = (c.colored_tet_order.cpu().numpy(), np.asarray(c.color_offsets))
  otraj, _, _ = run_oracle_xpbd(d, coloring=col)
  pinned = d['invm'] == 0
  assert np.isfinite(traj).all()
  assert np.abs(traj - otraj).max() < 5e-5
  x0p = d['x0'] + (np.float32(1.0 / 300.0) ** 2) * d['gravity']
  assert np.abs(traj[-1][pinned] - x0p[pinned]).max() < 1e-6
  d.update(kw_youngs_modulus=np.array(1e5), kw_poissons_ratio=np.array(0.3),
           kw_n_iterations=np.array(2), kw_method=np.array('color'))
  for k in ('kw_hydro_alpha', 'kw_devia_alpha'):
    d.pop(k)
  vtraj, _ = gpu_vbd(cuda, d)
  assert np.isfinite(vtraj).all()
