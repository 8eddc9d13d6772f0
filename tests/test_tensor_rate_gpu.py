"""The tcgen05 rate kernel behind bench.py's tensor workload runs real MMAs.

nexus_tensor_tile runs the kernel of nexus_tensor_rate on one CTA and copies
its tensor-memory accumulator out through tcgen05.ld.  With small-integer
operands every product and sum is exact in bf16 / e4m3 and the f32
accumulator, so the result must equal rounds * A . B^T word for word: this
pins the shared-memory descriptors, the instruction descriptor's shape and
formats, the accumulate flag and the tensor-memory lane layout that the rate
depends on.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BF16 = {-2: 0xC000, -1: 0xBF80, 0: 0x0000, 1: 0x3F80, 2: 0x4000}
E4M3 = {-2: 0xC0, -1: 0xB8, 0: 0x00, 1: 0x38, 2: 0x40}


def _encode(v, table, dtype):
    lut = np.zeros(5, dtype=dtype)
    for k, w in table.items():
        lut[k + 2] = w
    return lut[v + 2]


@pytest.mark.parametrize("kind", [0, 1], ids=["bf16", "e4m3"])
@pytest.mark.parametrize("rounds", [1, 3])
def test_tensor_tile_exact(cuda, kind, rounds):
    import nexus_gb300 as ng
    rng = np.random.default_rng(11 + 7 * kind + rounds)
    k = 64 if kind == ng.TENSOR_BF16 else 128        # 128 bytes of K per row
    a = rng.integers(-2, 3, size=(128, k))
    b = rng.integers(-2, 3, size=(256, k))
    table, dt = (BF16, np.uint16) if kind == ng.TENSOR_BF16 else (E4M3, np.uint8)
    d = ng.tensor_tile(kind, _encode(a, table, dt), _encode(b, table, dt), rounds)
    want = (rounds * (a @ b.T)).astype(np.float32)
    assert np.array_equal(d, want)


@pytest.mark.parametrize("kind", [0, 1], ids=["bf16", "e4m3"])
def test_tensor_rate_runs(cuda, kind):
    import nexus_gb300 as ng
    flops, ms = ng.tensor_rate(kind, 2000)
    # 152 SMs x 2000 x 4 MMAs of 2 * 128 * 256 * K FLOP: a positive, finite rate
    assert ms > 0
    assert 1e13 < flops < 1e17


def test_tensor_rate_rejects_bad_arguments(cuda):
    import nexus_gb300 as ng
    with pytest.raises(ng.NexusError):
        ng.tensor_rate(2, 10)
    with pytest.raises(ng.NexusError):
        ng.tensor_rate(0, 0)
