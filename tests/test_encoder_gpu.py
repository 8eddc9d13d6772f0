"""CKKS encoder parity: the engine's encode/decode against SEAL's own outputs."""
import numpy as np
import pytest

from tests.golden_data import load
from tests.util import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    return load()


@pytest.fixture(scope="module")
def ctx(g, cuda):
    from nexus_gb300 import Context
    return Context(int(g["log_n"]), [int(q) for q in g["moduli"]])


def _enc(ctx, values, scale, limbs):
    import torch
    out = torch.empty((limbs, ctx.n), dtype=torch.int64, device="cuda")
    ctx.encode(values, scale, limbs, out)
    return to_host(out)


def test_encode_real(g, ctx):
    assert np.array_equal(_enc(ctx, g["values_p"], 2.0 ** 30, 2), g["pt"])


def test_encode_complex(g, ctx):
    assert np.array_equal(_enc(ctx, g["values_c"], 2.0 ** 35, 2), g["pt_complex"])


def test_encode_short_vector_one_limb(g, ctx):
    assert np.array_equal(_enc(ctx, g["values_p"][:100], 2.0 ** 20, 1), g["pt_short"])


def test_encode_scalar(g, ctx):
    for v, sc, want in zip(g["scalar_vals"], g["scalar_scales"], g["scalar_pts"]):
        assert np.array_equal(ctx.encode_scalar(float(v), float(sc), 2), want), (v, sc)


def test_decode(g, ctx):
    got = ctx.decode(to_dev(g["pt"]), 2.0 ** 30)
    assert np.array_equal(got, g["decoded"])
    assert np.max(np.abs(got.real - g["values_p"])) < 1e-6


def test_encode_rejects_out_of_range(ctx):
    import torch
    from nexus_gb300 import NexusError
    out = torch.empty((2, ctx.n), dtype=torch.int64, device="cuda")
    with pytest.raises(NexusError, match="scale out of bounds"):
        ctx.encode(np.ones(4), 2.0 ** 95, 2, out)
    with pytest.raises(NexusError, match="too large"):
        ctx.encode(np.ones(ctx.n), 2.0 ** 30, 2, out)


def test_encode_n65536_root_table(cuda):
    """N = 2^16 pins every 2^17-th root of unity used by the FFT."""
    import torch
    from nexus_gb300 import Context
    from pathlib import Path
    d = np.load(Path(__file__).parent / "golden" / "ckks_encode_n65536.npz")
    ctx = Context(int(d["log_n"]), [int(q) for q in d["moduli"]])
    out = torch.empty((2, ctx.n), dtype=torch.int64, device="cuda")
    ctx.encode(d["values"], 2.0 ** 40, 2, out)
    assert np.array_equal(to_host(out), d["pt"])
    assert np.array_equal(ctx.decode(out, 2.0 ** 40), d["decoded"])
