"""The autotuner (nexus_autotune) picks launch parameters from its candidate
sets, and no choice changes a word: key switches and NTTs under the tuned,
the smallest and the largest settings, in both forms of the forward NTT,
give the oracle's words."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.util import to_dev, to_host

pytestmark = pytest.mark.gpu

LOG_N = 16
N = 1 << LOG_N


def test_autotune_choice_and_words(cuda):
    import torch
    from nexus_gb300 import Context
    qs = po.create_coeff_modulus(N, [51, 46, 46, 46, 51, 51, 51, 51])
    ctx = Context(LOG_N, qs)
    oc = po.OracleContext(LOG_N, qs)
    assert ctx.tuning() == {"ntt_prefetch_waves": 3, "ks_inner_ctas_per_sm": 0, "ntt_form": 0}
    t = ctx.autotune(7, 2, reps=2)
    assert t["ntt_prefetch_waves"] in (0, 1, 2, 3, 4) and t["ks_inner_ctas_per_sm"] in (0, 4, 8, 16)
    assert t["ntt_form"] in (0, 1, 2) and t["ms_per_call"] > 0
    assert ctx.tuning() == {k: t[k] for k in ("ntt_prefetch_waves", "ks_inner_ctas_per_sm", "ntt_form")}
    rng = np.random.default_rng(9)
    l = 7
    ct = po.random_residues(rng, (2, l, N), qs[:l])
    tgt = po.random_residues(rng, (1, l, N), qs[:l])[0]
    key = po.random_residues(rng, (len(qs) - 1, 2, len(qs), N), qs)
    want = oc.switch_key(ct, tgt, key)
    want_ntt = oc.ntt(ct, 0, l)
    for setting in (None, (0, 0, 0), (4, 16, 1), (1, 4, 1), (1, 4, 0), (1, 0, 2), (3, 8, 2)):
        if setting is not None:
            ctx.set_tuning(*setting[:2])
            ctx.set_ntt_form(setting[2])
        d = to_dev(ct)
        ctx.switch_key(d, to_dev(tgt), to_dev(key))
        torch.cuda.synchronize()
        assert np.array_equal(to_host(d), want), setting
        x = to_dev(ct)
        ctx.ntt_forward(x, 0, l)
        torch.cuda.synchronize()
        assert np.array_equal(to_host(x), want_ntt), setting
