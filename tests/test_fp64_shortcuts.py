"""Properties the FP64 pass-A shortcuts rely on, checked on the CPU with IEEE
double arithmetic (numpy, no fused multiply-add, the oracle's arithmetic).

1. The limiter value min(1, (bound - u) / delt2) (gpu_solver.cu:456-494; bound
   = Umax for delt2 > 0, Umin for delt2 < 0, so bound - u has delt2's sign or
   is zero) is exactly 1 whenever |bound - u| >= |delt2|: the GPU skips those
   divisions and shares the rest out over the warp.
2. The magnitude comparison on bit patterns (sign bit cleared, as unsigned
   64-bit integers) orders finite doubles like |x| < |y|, and puts a NaN
   above every finite value (so a NaN delt2 still takes the division path).
3. The face spectral radius (gpu_solver.cu:385-454, the oracle's operation
   order) is bitwise symmetric in its two states and in the sign of the face
   vector, so one evaluation per interior face serves both cells."""
import numpy as np


def _abs_bits(x):
    return np.asarray(x, np.float64).view(np.uint64) & np.uint64(0x7FFFFFFFFFFFFFFF)


def test_limiter_quotient_is_one_when_skipped():
    rng = np.random.default_rng(3)
    n = 200000
    u = rng.normal(size=n) * 10.0 ** rng.integers(-3, 3, n)
    delt2 = rng.normal(size=n) * 10.0 ** rng.integers(-8, 1, n)
    # bound on delt2's side of u, sometimes far, sometimes within one ulp
    gap = np.abs(delt2) * rng.choice([0.5, 0.999999, 1.0, 1.0000001, 2.0, 1e3], n)
    bound = np.where(delt2 > 0, u + gap, u - gap)
    num = bound - u
    with np.errstate(divide="ignore", invalid="ignore"):
        phi = np.fmin(num / delt2, 1.0)
    skip = (delt2 != 0) & ~(_abs_bits(num) < _abs_bits(delt2))
    assert skip.sum() > n // 4 and (~skip).sum() > n // 10
    assert np.all(phi[skip] == 1.0)


def test_magnitude_order_on_bits():
    rng = np.random.default_rng(4)
    x = rng.normal(size=100000) * 10.0 ** rng.integers(-300, 300, 100000)
    y = rng.normal(size=100000) * 10.0 ** rng.integers(-300, 300, 100000)
    x[:10] = 0.0
    x[10:20] = -0.0
    y[20:30] = np.inf
    assert np.array_equal(_abs_bits(x) < _abs_bits(y), np.abs(x) < np.abs(y))
    nan = np.float64(np.nan)
    assert np.all(_abs_bits(x[np.isfinite(x)]) < _abs_bits(nan))


def _spectral_radius(a, b, vx, vy, g):
    rou = (a[0] + b[0]) * 0.5
    u = (a[1] + b[1]) / rou * 0.5
    v = (a[2] + b[2]) / rou * 0.5
    ee = (a[3] + b[3]) * 0.5 / rou - (u * u + v * v) * 0.5
    vc = u * vx + v * vy
    p = rou * ee * (g - 1.0)
    cs = np.sqrt((g * p / rou) * (vy * vy + vx * vx))
    return np.abs(vc) + cs


def test_spectral_radius_is_bitwise_symmetric():
    rng = np.random.default_rng(5)
    n = 100000
    rho_a, rho_b = rng.uniform(0.2, 2.0, n), rng.uniform(0.2, 2.0, n)
    ua, ub = rng.normal(size=(2, n))
    va, vb = rng.normal(size=(2, n))
    ea = rho_a * (2.5 + 0.5 * (ua * ua + va * va)) + rng.uniform(0, 1, n)
    eb = rho_b * (2.5 + 0.5 * (ub * ub + vb * vb)) + rng.uniform(0, 1, n)
    a = np.stack([rho_a, rho_a * ua, rho_a * va, ea])
    b = np.stack([rho_b, rho_b * ub, rho_b * vb, eb])
    vx, vy = rng.normal(size=(2, n)) * 1e-2
    g = 1.4
    left = _spectral_radius(a, b, vx, vy, g)
    right = _spectral_radius(b, a, -vx, -vy, g)  # the other cell: states swapped, face vector negated
    assert np.array_equal(left.view(np.uint64), right.view(np.uint64))
