"""Checkpoint / resume and merging of GPU ensembles: a resumed job and a
merge of shards give the same bits as one uninterrupted ensemble."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from pypercolate_gb300 import _native as nat
    nat.lib_handle()
    return nat


PS = np.linspace(0.3, 0.7, 41)


def make():
    from pypercolate_gb300.ensemble import Ensemble
    return Ensemble('grid', 24, PS, precision='fp32', micro=True)


def bits(ens):
    st = ens.state()
    out = [st['count'], st['mean'], st['m2']]
    if st['micro'] is not None:
        out += [st['micro'][k] for k in sorted(st['micro'])]
    return [np.asarray(a).tobytes() for a in out]


def test_resume_is_bit_identical(gpu, tmp_path):
    from pypercolate_gb300 import store
    ref = make()
    for run0 in (0, 300, 600):
        ref.run(min(300, 700 - run0), key=5, run0=run0)
    path = str(tmp_path / 'ck.npz')
    # three "jobs", each allowed one batch, then one that finds nothing to do
    for expect_done in (False, False, True):
        ens, done = store.run_checkpointed(path, make, 700, 300, key=5, max_batches=1)
        assert done == expect_done
    ens, done = store.run_checkpointed(path, make, 700, 300, key=5, max_batches=1)
    assert done and ens.ledger == ref.ledger
    assert bits(ens) == bits(ref)
    assert bits(type(ens).load(path)) == bits(ref)
    np.testing.assert_array_equal(ens.canonical_averages(), ref.canonical_averages())
    m_ens, m_ref = ens.microcanonical_averages(), ref.microcanonical_averages()
    for k in m_ref:
        np.testing.assert_array_equal(m_ens[k], m_ref[k])
    # a checkpoint of another lattice is refused, not merged into
    from pypercolate_gb300.ensemble import Ensemble
    with pytest.raises(ValueError, match='different ensemble'):
        store.run_checkpointed(path, lambda: Ensemble('grid', 25, PS, micro=True), 700, 300, key=5)
    assert os.listdir(tmp_path) == ['ck.npz']


def test_merge_of_shards_equals_one_ensemble(gpu):
    whole = make()
    whole.run(400, key=9, run0=0)
    whole.run(250, key=9, run0=400)
    a = make().run(400, key=9, run0=0)
    b = make().run(250, key=9, run0=400)
    a.merge(b)
    assert bits(a) == bits(whole)
    # merging a saved state (dict) works the same way
    c = make().run(400, key=9, run0=0)
    c.merge(b.state())
    assert bits(c) == bits(whole)
    with pytest.raises(ValueError, match='twice'):
        a.merge(make().run(10, key=9, run0=640))
    from pypercolate_gb300.ensemble import Ensemble
    with pytest.raises(ValueError, match='differ'):
        a.merge(Ensemble('grid', 24, PS[:-1], micro=True))


def test_merge_matches_bond_reduce_of_rows(gpu):
    """The device merge agrees with bond_reduce on the reference's rows."""
    from pypercolate_gb300 import hpc
    a = make().run(300, key=2, run0=0)
    b = make().run(500, key=2, run0=300)
    rows = hpc.bond_reduce(a.canonical_averages(), b.canonical_averages())
    a.merge(b)
    got = a.canonical_averages()
    assert np.all(got['number_of_runs'] == 800)
    for f in got.dtype.names[1:]:
        np.testing.assert_allclose(got[f], rows[f], rtol=1e-12, atol=1e-12)


def test_state_of_other_models_round_trips(gpu, tmp_path):
    """Site percolation and torus wrapping ensembles (micro on and off) keep
    their model in the checkpoint, resume and merge like bond ensembles."""
    from pypercolate_gb300 import store
    from pypercolate_gb300.ensemble import Ensemble
    for kw in (dict(kind='torus', length=12, model='site', wrap='both', micro=True),
               dict(kind='grid', length=10, model='site', micro=False),
               dict(kind='torus', length=9, model='bond', wrap='x', micro=False)):
        make = lambda: Ensemble(kw['kind'], kw['length'], PS, micro=kw['micro'],  # noqa: E731
                                model=kw['model'], wrap=kw.get('wrap', 'either'))
        whole = make().run(120, key=4, run0=0).run(80, key=4, run0=120)
        path = str(tmp_path / ('%s_%s.npz' % (kw['kind'], kw['model'])))
        ens, done = store.run_checkpointed(path, make, 200, 120, key=4, max_batches=1)
        assert not done
        ens, done = store.run_checkpointed(path, make, 200, 120, key=4)
        assert done
        assert bits(ens) == bits(whole)
        loaded = Ensemble.load(path)
        assert (loaded.model, loaded.wrap, loaded.kind) == (kw['model'], kw.get('wrap', 'either'),
                                                           kw['kind'])
        # a bond ensemble of the same lattice is a different ensemble
        if kw['model'] == 'site':
            with pytest.raises(ValueError):
                loaded.merge(Ensemble(kw['kind'], kw['length'], PS, micro=kw['micro']))


def test_host_merge_of_states_matches_device_merge(gpu):
    """distributed.merge_states (numpy, for a coordinator without a GPU)
    gives the device merge's result (Ensemble.merge: nz_canonical_merge,
    nz_micro_merge): canonical and micro M2 to 1e-14, exact sums and counts
    equal."""
    from pypercolate_gb300.distributed import merge_states
    shards = []
    for run0, n in ((0, 200), (200, 150), (350, 77)):
        e = make()
        e.run(n, key=5, run0=run0)
        shards.append(e)
    states = [e.state() for e in shards]
    dev = shards[0]
    for e in shards[1:]:
        dev.merge(e)
    want = dev.state()
    got = merge_states(states)
    assert int(got['count'][0]) == int(want['count'][0]) == 427
    np.testing.assert_allclose(got['mean'], want['mean'], rtol=1e-14, atol=1e-300)
    np.testing.assert_allclose(got['m2'], want['m2'], rtol=1e-14, atol=1e-12)
    for k in ('count', 'span_count', 'sum_lo', 'sum_hi'):
        assert np.array_equal(np.asarray(got['micro'][k]), np.asarray(want['micro'][k])), k
    np.testing.assert_allclose(got['micro']['m2'], want['micro']['m2'], rtol=1e-14, atol=1e-9)


def test_merged_ensemble_of_one_rank_is_the_rank_itself(gpu):
    """distributed.merged_ensemble -- the gather and device merge that a
    multi-GPU job runs once after its runs -- in a one-rank gloo group gives
    back the rank's own state bit for bit (the N > 1 exchange is covered on
    CPU by tests/test_distributed.py)."""
    import socket
    import torch.distributed as dist
    from pypercolate_gb300.distributed import merged_ensemble
    sock = socket.socket()
    sock.bind(('127.0.0.1', 0))
    port = sock.getsockname()[1]
    sock.close()
    dist.init_process_group('gloo', init_method='tcp://127.0.0.1:%d' % port, rank=0, world_size=1)
    try:
        ens = make()
        ens.run(150, key=9, run0=0)
        merged = merged_ensemble(ens)
        assert bits(merged) == bits(ens)
        assert merged.ledger == ens.ledger
    finally:
        dist.destroy_process_group()
