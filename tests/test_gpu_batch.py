"""Batched commutators (imsrg_batch_*: 64 pairs of uneven size in one CUDA
graph, the 64-pair configuration with emax drawn from {2..6}) against the same
commutators evaluated one by one and against the C oracle.  The grouped
products split every pair's operands into the same digits as the pair's own
plan, so the only difference allowed against the one-by-one results is the
order of the zero-body atomic sums: 1e-14 relative."""
import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import rel_errors
from oracle import Oracle

pytestmark = pytest.mark.gpu


def make_pairs(n, seed, emaxes=(2, 3, 4, 5, 6)):
    rng = np.random.Generator(np.random.PCG64(seed))
    es = [int(e) for e in rng.choice(emaxes, size=n)]
    spaces = {}
    pairs = []
    for i, e in enumerate(es):
        ms = ig.ModelSpace(e, "O16", "O16")  # one space per pair: pairs run concurrently
        spaces[i] = ms
        dX, dY, dZ = ig.DeviceOperator(ms, 1), ig.DeviceOperator(ms, -1), ig.DeviceOperator(ms, 1)
        dX.fill_random(1000 + 2 * i)
        dY.fill_random(1001 + 2 * i)
        pairs.append((dX, dY, dZ))
    return es, pairs


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_batch_matches_single_launches(prec):
    es, pairs = make_pairs(64, 4, )
    assert set(es) == {2, 3, 4, 5, 6}
    refs = []
    for dX, dY, dZ in pairs:
        ig.Commutator.device_commutator(dX, dY, dZ, prec)
        refs.append(dZ.download())
    for _, _, dZ in pairs:
        dZ.zero()
    b = ig.CommutatorBatch(pairs, prec)
    n, branches, grouped, nodes = b.info()
    # one chain of launches per emax: at least the ten kernels of a commutator each
    assert (n, branches) == (64, 64) and 5 * 10 <= nodes < 64 * 10
    # both forms: the products (and every other kernel) of the pairs of each
    # emax run as one launch
    assert grouped == 5
    for _, _, dZ in pairs:
        dZ.zero()
    for _ in range(2):
        b.launch()
    b.sync()
    for (dX, dY, dZ), ref in zip(pairs, refs):
        assert max(rel_errors_any(dZ, ref)) < 1e-14


def rel_errors_any(dZ, ref):
    Z = dZ.download()
    scale = max(np.linalg.norm(ref), 1e-300)
    return [np.linalg.norm(Z - ref) / scale]


def test_batch_vs_oracle_shared_spaces():
    # pairs sharing a model space run in order on one graph branch
    emaxes = [2, 4, 2, 4, 3]
    spaces = {e: ig.ModelSpace(e, "O16", "O16") for e in set(emaxes)}
    oracles = {e: Oracle(e) for e in set(emaxes)}
    pairs, inputs = [], []
    for i, e in enumerate(emaxes):
        o = oracles[e]
        X = o.ms.random_operator(300 + i, True)
        Y = o.ms.random_operator(400 + i, False)
        dX, dY, dZ = ig.DeviceOperator(spaces[e], 1), ig.DeviceOperator(spaces[e], -1), ig.DeviceOperator(spaces[e], 1)
        dX.upload(X)
        dY.upload(Y)
        pairs.append((dX, dY, dZ))
        inputs.append((e, X, Y))
    b = ig.CommutatorBatch(pairs, "fp64")
    assert b.info()[:3] == (5, 3, 0)
    for _, _, dZ in pairs:
        dZ.zero()
    b.launch()
    b.sync()
    for (e, X, Y), (_, _, dZ) in zip(inputs, pairs):
        R = oracles[e].commutator(X, Y, 1, -1)
        assert max(rel_errors(oracles[e].ms, dZ.download(), R)) < 1e-12


def test_batch_rejects_repeated_z():
    ms = ig.ModelSpace(2, "O16", "O16")
    dX, dY, dZ = ig.DeviceOperator(ms, 1), ig.DeviceOperator(ms, -1), ig.DeviceOperator(ms, 1)
    with pytest.raises(ig.IMSRGError):
        ig.CommutatorBatch([(dX, dY, dZ), (dY, dX, dZ)], "fp64")
