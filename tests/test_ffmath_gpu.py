"""The float-float evaluations that stand for the reference's double
sub-expressions must give the double evaluation's float bit for bit whenever
their rounding test lets them answer (otherwise the double path runs).
Unary functions are checked on every float of their working range, the
others on 2^27-2^28 hashed inputs each; the fast paths must answer almost
always."""
import pytest

pytestmark = pytest.mark.gpu

(ASIN, ATAN2, PHI, ADD_SQRT, ADD_SQRT3, PHI_MPI_PI, ADD_PI, PT, MULS, QSQ, SIN, COS, ATAN, HYPOT, T15, MULS1,
 PHI_APPROX, ASIN_APPROX, TAN, TAN_OVER, PHI_FAST) = range(21)


@pytest.fixture(scope="module")
def gpu():
    from sdl_gb300 import Chain, build
    build.build()
    return Chain(0)


def _bits(x):
    import struct
    return struct.unpack("<I", struct.pack("<f", x))[0]


@pytest.mark.parametrize("fn,lo,hi,min_answered,signs", [
    (ASIN, 2.0 ** -30, 0.95, 0.999, 2),        # every float of the std::asin arguments
    (PHI_MPI_PI, 3.1415927, 9.0, 0.999, 2),    # every float the loop's first step handles
    (ADD_PI, 2.0 ** -20, 3.1415925, 0.99, 2),  # M_PI + atan2 result
    (SIN, 2.0 ** -30, 8.0, 0.999, 2),          # every float of the angles the strip shift uses
    (COS, 2.0 ** -30, 8.0, 0.999, 2),
    (ATAN, 2.0 ** -40, 2.0 ** 40, 0.999, 2),
    # every float of the hits' asin angles asin(min(rt k, 0.95)) for rt above 0.2 cm
    (TAN, 2.0 ** -10, 1.2533, 0.999, 1),
    (TAN_OVER, 2.0 ** -10, 1.2533, 0.999, 1),
])
def test_unary_exhaustive(gpu, fn, lo, hi, min_answered, signs):
    n = _bits(hi) - _bits(lo) + 1
    for sign in (0, 0x80000000)[:signs]:
        r = gpu.math_check(fn, n, start=sign | _bits(lo), exhaustive=True)
        assert r["mismatches"] == 0, r
        assert r["answered"] >= min_answered * n, (r["answered"], n)


@pytest.mark.parametrize("fn,n,min_answered", [
    (ATAN2, 1 << 28, 0.99), (PHI, 1 << 27, 1.0), (ADD_SQRT, 1 << 27, 0.99), (ADD_SQRT3, 1 << 27, 0.99),
    (PT, 1 << 27, 0.99), (MULS, 1 << 27, 0.99), (MULS1, 1 << 27, 0.99), (QSQ, 1 << 27, 0.99),
    (HYPOT, 1 << 27, 0.99), (T15, 1 << 27, 0.99)])
def test_random_inputs(gpu, fn, n, min_answered):
    r = gpu.math_check(fn, n, seed=12345)
    assert r["mismatches"] == 0, r
    assert r["answered"] >= min_answered * n, (r["answered"], n)


def test_phase_b1_approximation_bounds(gpu):
    """Phase B1 decides from atan2f / asinf when a cut holds or fails by 1e-4;
    both approximations must stay within 2e-6 of the exact values (asinf on
    every float of the asin arguments, the directions on 2^28 hashed points)."""
    n = _bits(0.95) - _bits(2.0 ** -30) + 1
    for sign in (0, 0x80000000):
        r = gpu.math_check(ASIN_APPROX, n, start=sign | _bits(2.0 ** -30), exhaustive=True)
        assert r["mismatches"] == 0 and r["answered"] == n, r
    r = gpu.math_check(PHI_APPROX, 1 << 28, seed=777)
    assert r["mismatches"] == 0 and r["answered"] == 1 << 28, r
    # the enumeration's polynomial direction (phi_fast): within 2.5e-6
    r = gpu.math_check(PHI_FAST, 1 << 28, seed=778)
    assert r["mismatches"] == 0 and r["answered"] == 1 << 28, r
