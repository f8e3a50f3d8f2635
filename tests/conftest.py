import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, 'tests', 'golden')
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)


def pytest_configure(config):
  config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')
  config.addinivalue_line('markers', 'slow: takes more than a few seconds')


def golden(name):
  return np.load(os.path.join(GOLDEN, name))


STEP_CASES = ['box5x4x5_mu1e5', 'box5x4x5_ls', 'cube6_mu3e4']


def step_fixture_names():
  out = []
  for c in STEP_CASES:
    for suffix in ('', '_cgalias'):
      if os.path.exists(os.path.join(GOLDEN, f'step_{c}{suffix}.npz')):
        out.append(f'step_{c}{suffix}.npz')
  return out


def solver_kwargs(z):
  kw = dict(mu=float(z['param_mu']), damp=float(z['param_damp']))
  if 'param_maxiter' in z.files:
    kw['maxiter'] = int(z['param_maxiter'])
  return kw


@pytest.fixture(scope='session')
def cuda():
  torch = pytest.importorskip('torch')
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from controllable_pbd_3d_gb300 import _native
  _native.lib()
  return torch


@pytest.fixture(scope='session')
def cuda_or_cpu():
  """'cuda' where a GPU is visible, else 'cpu' (host-only code paths)."""
  torch = pytest.importorskip('torch')
  return 'cuda' if torch.cuda.is_available() else 'cpu'
