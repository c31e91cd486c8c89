"""CPU tests of the oracle itself: it must reproduce the reference's golden
vectors (pinning) before anything is checked against it."""
import numpy as np
import pytest

import oracle as O
from helpers import as_complex, cases, read_bin

# Tight bound for the FP64 oracle against the float32 goldens: the goldens
# are torch.fft complex64 results, so they carry float32 rounding (~1e-7).
GOLD_REL = 2e-6


def _check_gold(out, gold, c):
    ok, det = O.comparison_details(out, gold, c["atol"], c["rtol"])
    assert ok, det
    assert det["rel_l2"] < GOLD_REL, det


@pytest.mark.parametrize("c", cases("fft1_d"), ids=lambda c: c["name"])
def test_oracle_pins_fft1_d(c):
    n, b = c["n"], c["batch"]
    x = as_complex(read_bin("fft1_d", c["files"]["input"]))
    gold = read_bin("fft1_d", c["files"]["golden"])
    if c.get("roundtrip"):
        fwd = O.c2c(x.reshape(b, n), -1)
        gfwd = read_bin("fft1_d", c["files"]["golden_forward"])
        _check_gold(fwd, gfwd, c)
        out = O.c2c(fwd, +1)
    elif c.get("vertical"):
        out = O.c2c_vertical(x.reshape(n, b), -1 if c["forward"] else +1)
    else:
        out = O.c2c(x.reshape(b, n), -1 if c["forward"] else +1)
    _check_gold(out, gold, c)


@pytest.mark.parametrize("c", cases("rfft1_d"), ids=lambda c: c["name"])
def test_oracle_pins_rfft1_d(c):
    n, b = c["n"], c["batch"]
    x = read_bin("rfft1_d", c["files"]["input"]).reshape(b, n)
    gold = read_bin("rfft1_d", c["files"]["golden"])
    _check_gold(O.r2c(x), gold, c)


@pytest.mark.parametrize("c", cases("irfft1_d"), ids=lambda c: c["name"])
def test_oracle_pins_irfft1_d(c):
    n, b = c["n"], c["batch"]
    X = as_complex(read_bin("irfft1_d", c["files"]["input"])).reshape(b, n // 2 + 1)
    gold = read_bin("irfft1_d", c["files"]["golden"])
    _check_gold(O.c2r(X, n), gold, c)


@pytest.mark.parametrize("c", cases("fft2_d"), ids=lambda c: c["name"])
def test_oracle_pins_fft2_d(c):
    nx, ny, b = c["fft_x"], c["fft_y"], c["batch"]
    x = as_complex(read_bin("fft2_d", c["files"]["input"])).reshape(b, nx, ny)
    gold = read_bin("fft2_d", c["files"]["golden"])
    _check_gold(O.c2c_2d(x, -1 if c["forward"] else +1), gold, c)


def test_known_answer_n2():
    """N=2 example of the reference's test guide: {1+2j, 3+4j} -> {4+6j, -2-2j}."""
    out = O.c2c(np.array([[1 + 2j, 3 + 4j]]), -1)
    assert np.array_equal(out, np.array([[4 + 6j, -2 - 2j]]))


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 12, 97, 210, 1000, 4096, 4099])
def test_oracle_against_direct_dft(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    bins = np.unique(np.array([0, 1, n // 3, n // 2, n - 1]) % n)
    for sign in (-1, 1):
        full = O.c2c(x[None], sign)[0]
        direct = O.dft_bins(x, bins, sign)
        assert np.abs(full[bins] - direct).max() <= 1e-12 * max(1.0, np.abs(direct).max()) * n


@pytest.mark.parametrize("n", [1, 2, 6, 7, 8, 15, 64, 1000, 1023, 3000])
def test_real_oracles_consistent_with_complex(n):
    rng = np.random.default_rng(n + 7)
    x = rng.standard_normal((3, n))
    X = O.r2c(x)
    full = O.c2c(x.astype(np.complex128), -1)
    assert np.abs(X - full[:, : n // 2 + 1]).max() < 1e-11 * n
    y = O.c2r(X, n)
    assert np.abs(y - n * x).max() < 1e-10 * n


def test_port_matches_oracle():
    """The FP32 port of the reference path used as the CPU baseline."""
    rng = np.random.default_rng(3)
    for n in (64, 1500, 3000, 1024):
        x = rng.standard_normal((4, n)).astype(np.float32)
        e = O.errors(O.port_r2c(x), O.r2c(x))
        assert e["rel_l2"] < 1e-5, (n, e)
        X = O.r2c(x)
        e = O.errors(O.port_c2r(X.astype(np.complex64), n), O.c2r(X, n))
        assert e["rel_l2"] < 1e-5, (n, e)
    z = (rng.standard_normal((2, 4096)) + 1j * rng.standard_normal((2, 4096))).astype(np.complex64)
    assert O.errors(O.port_c2c(z), O.c2c(z))["rel_l2"] < 1e-5


def test_ordered_factorize_matches_reference_examples():
    # examples verified against the reference's own helper
    assert O.ordered_factorize(4096) == [2] * 12
    assert O.ordered_factorize(3000) == [2, 2, 2, 3, 5, 5, 5]
    assert O.ordered_factorize(46200) == [2, 2, 2, 3, 5, 5, 7, 11]
    assert O.choose_radix(True, 4096) == 2
    assert O.choose_radix(True, 3000) == -2
    assert O.choose_radix(False, 4096) == -2
    assert O.choose_radix(True, 53 * 2) == -1


@pytest.mark.parametrize("radices", [[2], [4, 4], [16, 16, 16], [15, 10, 10], [8, 8, 8], [11, 5, 4], [37, 9, 3], [7, 2, 3]])
def test_stockham_index_maps_are_permutations(radices):
    """Each pass's read and write maps cover [0, L) exactly once (integers,
    bit-exact), and the passes compose to a natural-order DFT."""
    L = int(np.prod(radices))
    for read, write in O.stockham_index_maps(radices):
        assert np.array_equal(np.sort(read.reshape(-1)), np.arange(L))
        assert np.array_equal(np.sort(write.reshape(-1)), np.arange(L))
    rng = np.random.default_rng(L)
    x = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    assert np.abs(O.stockham_simulate_exact(x, radices) - O.c2c(x[None])[0]).max() < 1e-10 * L


def test_long_row_oracle_agrees_with_c_oracle():
    """The numpy FP64 path used for the longest reference rows (2^23-2^27)
    agrees with the C oracle to FP64 rounding at 2^20 and an odd length."""
    rng = np.random.default_rng(11)
    for n in (1 << 20, 999999):
        x = rng.standard_normal((1, n))
        a, b = O.r2c(x), O.r2c_long_rows(x)
        assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-13


@pytest.mark.parametrize("shape", [(1, 8, 6), (2, 7, 10), (3, 16, 15), (1, 1, 5), (2, 5, 1), (1, 30, 64)])
def test_multidim_real_oracles_agree_with_numpy(shape):
    """The 2D real oracles (composed from the pinned 1D C oracle) agree with
    numpy's independent FP64 rfft2 / irfft2 to FP64 rounding, and the 2D C2C
    oracle with the pinned fft2_d oracle."""
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape)
    nx, ny = shape[-2:]
    X = O.r2c_2d(x)
    ref = np.fft.rfft2(x)
    assert np.abs(X - ref).max() < 1e-12 * nx * ny
    # C2R of a general half spectrum: only the real parts of the ny=0 and
    # ny/2 bins of the column-transformed data enter (numpy's convention)
    Y = rng.standard_normal(X.shape) + 1j * rng.standard_normal(X.shape)
    y = O.c2r_2d(Y, ny)
    assert np.abs(y - np.fft.irfft2(Y, s=(nx, ny)) * nx * ny).max() < 1e-11 * nx * ny
    assert np.abs(O.c2r_2d(X, ny) - nx * ny * x).max() < 1e-10 * nx * ny
    z = x + 1j * rng.standard_normal(shape)
    assert np.abs(O._c2c_axis(O.c2c(z, -1), -2, -1) - O.c2c_2d(z, -1)).max() < 1e-12 * nx * ny


@pytest.mark.parametrize("shape", [(2, 3, 4), (5, 1, 7), (8, 8, 8), (1, 1, 1), (3, 30, 10)])
def test_3d_oracle_agrees_with_numpy(shape):
    rng = np.random.default_rng(sum(shape) + 1)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    n = int(np.prod(shape))
    assert np.abs(O.c2c_3d(x, -1) - np.fft.fftn(x)).max() < 1e-12 * n
    assert np.abs(O.c2c_3d(x, +1) - np.fft.ifftn(x) * n).max() < 1e-12 * n


@pytest.mark.parametrize("shape", [(2, 3, 4), (5, 1, 7), (4, 6, 8), (1, 1, 1), (3, 10, 9)])
def test_3d_real_oracles_agree_with_numpy(shape):
    rng = np.random.default_rng(sum(shape) + 2)
    x = rng.standard_normal(shape)
    n = int(np.prod(shape))
    X = O.r2c_3d(x)
    assert np.abs(X - np.fft.rfftn(x)).max() < 1e-12 * n
    Y = rng.standard_normal(X.shape) + 1j * rng.standard_normal(X.shape)
    assert np.abs(O.c2r_3d(Y, shape[-1]) - np.fft.irfftn(Y, s=shape, axes=(0, 1, 2)) * n).max() < 1e-11 * n
