"""The seeded workload generators are deterministic: the same instances on
every machine (the integer splitmix64 stream, IEEE-exact float steps and the
log-uniform sizes in decimal arithmetic), pinned by digests of small
instances of every generator.  The GPU-marked twin checks the same digests on
the machine that runs the GPU tests."""
import hashlib

import numpy as np
import pytest

import workloads as W


def _digest(arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).astype("<i8").tobytes())
    return h.hexdigest()[:16]


def _inst(i):
    return [i.lb, i.ub, i.op, i.x, i.y, i.z]


CASES = {
    "single_small_0": (lambda: _inst(W.single_small(0)), "97c4b9f07e353f57"),
    "plain_spec_3": (lambda: _inst(W.plain(2000, 6000, 1000, 3, variant="spec")), "244b271c1bdb32f7"),
    "chain_1": (lambda: _inst(W.add_chain(W.plain(500, 1500, 10**6, 1), 200, 10**6, 1)), "7b8760c578c08a18"),
    "uneven_8": (lambda: sum((_inst(i) for i in W.uneven(8, 1000, 20000, 1)), []), "15c3e0900e128270"),
    "nodes_small": (lambda: (lambda r: _inst(r[0]) + list(r[1:]))(W.nodes(2000, 8000, 64, 2)), "504d12c016261757"),
    "pc_mix_4": (lambda: list(W.pc_mix(3000, 2000, seed=4)), "cd39d7d632c37e65"),
}


def _check(name):
    make, want = CASES[name]
    got = _digest(make())
    assert got == want, (name, got)


@pytest.mark.parametrize("name", sorted(CASES))
def test_workload_digests(name):
    _check(name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_workload_digests_on_gpu_host(name):
    _check(name)


def test_uneven_sizes_log_uniform():
    sizes = W.uneven_sizes(4096, 1000, 200_000, 5)
    assert sizes.min() >= 1000 and sizes.max() < 200_000
    # log-uniform: each of the 4 equal ranges of log(size) holds about a quarter
    q = np.floor(4 * np.log(sizes / 1000) / np.log(200)).astype(int)
    assert all(0.2 < (q == k).mean() < 0.3 for k in range(4))
    # the same sizes numpy's exp / log give on this machine (the instances of
    # every benchmark run so far)
    u = W.Rng(5, 202).random(4096)
    ref = np.floor(np.exp(np.log(1000) + u * (np.log(200_000) - np.log(1000)))).astype(np.int64)
    assert np.array_equal(sizes, ref)
