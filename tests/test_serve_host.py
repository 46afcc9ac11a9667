"""CPU checks of the serving layer: request validation and admission sizes
are host logic (no device needed), the served workload generator has the
shapes of the load+RREF stream, and a server cannot start without a GPU."""
import ctypes
from math import comb

import numpy as np
import pytest

import oracle
from linac_gb300 import _lib, workloads
from linac_gb300.serving import SERVE_LOAD_RREF, SERVE_RREF, Server, _bind, lnc_serve_request


def _req(**kw):
    base = dict(kind=SERVE_RREF, dtype=_lib.LNC_U32, p=2**31 - 1, tol=0.0, m=100, n=120, host_in=1, ld_in=120,
                host_out=1, ld_out=120)
    base.update(kw)
    return lnc_serve_request(**base)


def _bytes(req):
    _bind()
    return int(_lib.lib().lnc_serve_request_bytes(ctypes.byref(req)))


def test_request_bytes_and_validation():
    ok = _bytes(_req())
    assert ok >= 2 * 100 * 120 * 4
    assert _bytes(_req(kind=7)) == -1
    assert _bytes(_req(p=2**31 - 2)) == -1          # not prime
    assert _bytes(_req(ld_in=10)) == -1             # ld < n
    assert _bytes(_req(ld_out=10)) == -1
    assert _bytes(_req(m=0)) == -1                  # empty
    assert _bytes(_req(host_out=None)) == -1
    assert _bytes(_req(dtype=_lib.LNC_U64, p=2**61 - 1)) >= 2 * 100 * 120 * 8
    load = _req(kind=SERVE_LOAD_RREF, host_in=None, host_bases=1, basis_len=12, host_lindices=1, degree=4)
    assert _bytes(load) >= ok + 100 * 12 * 4 + 120 * 4 * 4
    assert _bytes(_req(kind=SERVE_LOAD_RREF, host_in=None, host_bases=1, basis_len=0, host_lindices=1,
                       degree=4)) == -1


def test_served_workload_shapes_and_oracle_load():
    for d in range(3, 9):
        mono = workloads.monomial_indices(10, d)
        assert mono.shape == (min(comb(10 + d, d), 8000), d)
        assert len({tuple(r) for r in mono}) == mono.shape[0]
    rng = np.random.default_rng(0)
    p = workloads.random_prime_below(2**31, rng)
    assert 2**30 <= p < 2**31
    bases, lind = workloads.serve_load_request(rng, 3, p)
    assert bases.shape == (286 + 16, 12) and lind.shape == (286, 4)
    assert (bases[:, 0] == 1).all() and (bases[:, 11] > 0).all() and (bases < p).all()
    A = oracle.load_modp(bases, lind, p)
    # column of the monomial x_1 (indices 0, 0, 1): prefactor * x_1
    c = int(np.flatnonzero((lind[:, :3] == [0, 0, 1]).all(axis=1))[0])
    assert np.array_equal(A[:, c], (bases[:, 1].astype(np.uint64) * bases[:, 11]) % p)


@pytest.mark.skipif(_lib.device_count() > 0, reason="a GPU is present")
def test_server_needs_a_device():
    with pytest.raises(_lib.LinacGpuError):
        Server()
