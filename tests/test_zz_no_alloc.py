"""nexus_switch_key_noalloc: key switching with no device allocation.

Callers whose device memory belongs to another runtime's pool, or that may
not trigger the device-wide synchronisation of cudaMalloc/cudaFree, use this
entry point instead of nexus_switch_key.  Its temporaries live in a fixed
16 MiB device array inside the library.  This test checks, through the C
ABI, that two calls in a row give exactly the words nexus_switch_key gives
(integer results, so the tolerance is zero), and that a request larger than
the array is refused.  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from tests.util import to_dev, to_host

pytestmark = pytest.mark.gpu


def _noalloc():
    from nexus_gb300 import _lib
    f = _lib.lib().nexus_switch_key_noalloc
    return f


def _case(rng, qs, n, limbs):
    k = len(qs)
    ct = po.random_residues(rng, (2, limbs, n), qs[:limbs])
    tgt = po.random_residues(rng, (1, limbs, n), qs[:limbs])[0]
    key = po.random_residues(rng, (k - 1, 2, k, n), qs)
    return ct, tgt, key


@pytest.mark.parametrize("bits", [[60, 40, 40, 40, 40, 50, 60],    # the 64-bit product paths
                                  [50, 40, 40, 40, 40, 46, 50]])   # every prime < 2^52: the split paths
def test_noalloc_matches_switch_key_twice(cuda, bits):
    import torch
    from nexus_gb300 import Context, check
    log_n, n = 13, 1 << 13
    qs = po.create_coeff_modulus(n, bits)
    ctx = Context(log_n, qs)
    rng = np.random.default_rng(2025)
    f = _noalloc()
    for limbs in (6, 3):  # second call at another level reuses the same device array
        ct, tgt, key = _case(rng, qs, n, limbs)
        a = to_dev(ct)
        ctx.switch_key(a, to_dev(tgt), to_dev(key))
        b = to_dev(ct)
        check(f(ctx.handle, b.data_ptr(), limbs, to_dev(tgt).data_ptr(), to_dev(key).data_ptr(), None),
              "nexus_switch_key_noalloc")
        torch.cuda.synchronize()
        assert np.array_equal(to_host(b), to_host(a))


def test_noalloc_rejects_oversized_request(cuda):
    from nexus_gb300 import Context, _lib
    log_n, n = 16, 1 << 16
    qs = po.create_coeff_modulus(n, [60, 50, 50, 50, 50, 60])
    ctx = Context(log_n, qs)
    rng = np.random.default_rng(1)
    ct, tgt, key = _case(rng, qs, n, 4)  # 2^16 * (16 + 24 + 4) words > 2^21
    b = to_dev(ct)
    rc = _noalloc()(ctx.handle, b.data_ptr(), 4, to_dev(tgt).data_ptr(), to_dev(key).data_ptr(), None)
    assert rc != 0
    assert b"scratch words" in _lib.lib().nexus_last_error()
    assert np.array_equal(to_host(b), ct)  # refused before any work
