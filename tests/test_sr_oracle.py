"""The stochastic rounding of the SR storage forms, on the oracle (CPU): a
store lands on one of the two 16-bit values around the fp32 value, the one
above with probability equal to the distance from the one below (so the mean
over many hashes is the value itself), and it is reproducible."""
import numpy as np
import pytest

from oracle import oracle as O


def _neighbours_f16(v):
    """The fp16 values (in the stored scale 2^10) just below and above v."""
    s = np.float32(v) * np.float32(1024.0)
    lo = np.float16(s)
    if np.float32(lo) > s:
        lo = np.nextafter(lo, np.float16(-np.inf))
    hi = np.nextafter(lo, np.float16(np.inf)) if np.float32(lo) != s else lo
    return float(np.float32(lo)) / 1024.0, float(np.float32(hi)) / 1024.0


def _neighbours_bf16(v):
    b = np.array([v], np.float32).view(np.uint32)[0]
    lo = np.array([b & 0xFFFF0000], np.uint32).view(np.float32)[0]
    hi = np.array([(b & 0xFFFF0000) + 0x10000], np.uint32).view(np.float32)[0]
    if lo == np.float32(v):
        hi = lo
    return (float(lo), float(hi)) if v >= 0 else (float(hi), float(lo))


@pytest.mark.parametrize("storage,nb", [(O.F16SR, _neighbours_f16), (O.BF16SR, _neighbours_bf16)])
def test_sr_store_is_unbiased_between_neighbours(storage, nb):
    L = O.lib()
    rng = np.random.default_rng(3)
    for v in list(rng.uniform(-0.05, 0.05, 40)) + [1e-3, -2.5e-4, 0.0123456]:
        v = float(np.float32(v))
        lo, hi = nb(v)
        outs = np.array([L.orc_sr_store_f32(v, storage, L.orc_sr_cell_hash(c, 7), i)
                         for c in range(2000) for i in (1, 8)])
        assert np.all((outs == lo) | (outs == hi)), v
        if hi != lo:
            p_hi = (v - lo) / (hi - lo)
            assert abs(np.mean(outs == hi) - p_hi) < 0.04, (v, p_hi, np.mean(outs == hi))
            assert abs(outs.mean() - v) < 0.04 * (hi - lo) + 1e-12


def test_sr_store_is_reproducible_and_varies_with_step_cell_direction():
    L = O.lib()
    v = 0.0123456
    a = [L.orc_sr_store_f32(v, O.F16SR, L.orc_sr_cell_hash(c, s), i) for c in range(50) for s in (0, 1) for i in (0, 5)]
    b = [L.orc_sr_store_f32(v, O.F16SR, L.orc_sr_cell_hash(c, s), i) for c in range(50) for s in (0, 1) for i in (0, 5)]
    assert a == b and len(set(a)) == 2
    assert L.orc_sr_cell_hash(3, 0) != L.orc_sr_cell_hash(3, 1) != L.orc_sr_cell_hash(4, 1)


def test_sr_exactly_representable_values_stay():
    L = O.lib()
    for v in (0.0, 0.5 / 1024, -0.25 / 1024, 3.0 / 1024):
        for c in range(64):
            assert L.orc_sr_store_f32(v, O.F16SR, L.orc_sr_cell_hash(c, 2), 3) == np.float32(v)
    for v in (0.0, 0.5, -0.25):
        assert L.orc_sr_store_f32(v, O.BF16SR, L.orc_sr_cell_hash(1, 2), 3) == np.float32(v)
