import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, 'tests', 'golden')
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (sm_103a)')


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def golden_cases():
    """The reference's bond_microcanonical_statistics cases as dicts."""
    z = load_golden('hpc_cases.npz')
    out = []
    for ci in range(int(z['n_cases'])):
        pre = 'c%02d_' % ci
        L, seed, spanning, N, M = (int(x) for x in z[pre + 'meta'])
        case = dict(kind=str(z[pre + 'kind']), L=L, seed=seed, spanning=bool(spanning),
                    N=N, M=M)
        for k in ('eu', 'ev', 'side', 'perm', 'edge', 'max', 'moments', 'n'):
            case[k] = z[pre + k]
        if spanning:
            case['span'] = z[pre + 'span']
        out.append(case)
    return out


@pytest.fixture(scope='session')
def oracle():
    from oracle import oracle as O
    O.lib()
    return O
