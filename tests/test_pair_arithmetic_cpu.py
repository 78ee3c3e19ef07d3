"""The float-pair arithmetic of the mixed form, restated in numpy float32
(IEEE single precision, no fused multiply-add), as the step engine, the
kernel sequence's stage stencil and the true-stage Tsit5 use it:

* the state x (FP64) is carried as x = hi + lo with hi = fl32(x) and
  lo = fl32(x - hi);
* first differences of a stage state are formed as
  (hi_{i+1} - hi_i) + (lo_{i+1} - lo_i) in FP32 instead of taking the FP64
  difference and rounding it;
* each step adds an FP32 increment to the pair by a two-sum
  (s = hi + inc, the rounding error of s recovered exactly, folded into lo
  and renormalised).

The first must equal the rounded FP64 difference to FP32 rounding, the
second must track the FP64 state to about 2^-48 over many steps."""
import numpy as np

f32 = np.float32


def split(x):
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def pair_diff(hi, lo):
    return (hi[1:] - hi[:-1]) + (lo[1:] - lo[:-1])


def two_sum_add(hi, lo, inc):
    sm = hi + inc
    bb = sm - hi
    er = (hi - (sm - bb)) + (inc - bb)
    l2 = lo + er
    h2 = sm + l2
    return h2, l2 - (h2 - sm)


def test_pair_differences_match_rounded_fp64_differences():
    rng = np.random.default_rng(5)
    # a deflection profile of a few hundred metres with metre-scale
    # neighbour differences and a rounding-level tail
    x = np.cumsum(rng.normal(0.0, 1.0, 4096)) * 0.5 - 300.0 + rng.normal(0.0, 1e-9, 4096)
    hi, lo = split(x)
    assert np.all(hi.astype(np.float64) + lo.astype(np.float64) - x <= 1e-13 * np.abs(x).max())
    d_pair = pair_diff(hi, lo).astype(np.float64)
    d_ref = (x[1:] - x[:-1]).astype(np.float32).astype(np.float64)
    ulp = np.spacing(np.abs(d_ref).astype(np.float32)).astype(np.float64)
    # within one float32 ulp of the correctly rounded difference, plus the
    # pair's own representation error (2^-48 of |x|)
    assert np.all(np.abs(d_pair - d_ref) <= ulp + 2.0 ** -47 * np.abs(x).max())


def test_two_sum_steps_track_the_fp64_state():
    rng = np.random.default_rng(9)
    x = rng.normal(-200.0, 50.0, 2048)
    hi, lo = split(x)
    for _ in range(1000):
        inc = rng.normal(0.0, 0.05, x.size).astype(np.float32)   # one step's float increment
        x = x + inc.astype(np.float64)                             # the FP64 state update
        hi, lo = two_sum_add(hi, lo, inc)
    pair = hi.astype(np.float64) + lo.astype(np.float64)
    # each two-sum is exact up to the final renormalisation of lo: the pair
    # stays within a few 2^-48 of |x| after a thousand steps, far below the
    # FP32 rounding (2^-24) of any single difference
    assert np.abs(pair - x).max() <= 2.0 ** -40 * np.abs(x).max()
    assert np.all(np.abs(lo) <= np.spacing(np.abs(hi)))   # normalised: |lo| within one ulp of hi


def test_stage_state_differences_from_the_pair_and_the_previous_stage():
    """The stage state y = x + s (k - cm) differenced as the engine does:
    (pair diff of x) + s (k diff) in FP32 against the FP64 state
    differences, for RK4's stage scale at dt = 1 yr.  The FP32 sum of the
    two terms rounds relative to the terms, not to their (possibly
    cancelling) sum: the bound is a few ulp of the larger term."""
    rng = np.random.default_rng(13)
    n = 4096
    x = np.cumsum(rng.normal(0.0, 1.0, n)) * 0.5 - 300.0
    k = rng.normal(0.0, 1e-9, n).astype(np.float32)     # a stage RHS in m/s
    s = f32(0.5 * 1.0 * 31557600.0)                       # a h spy
    cm = f32(0.0)
    hi, lo = split(x)
    dx = pair_diff(hi, lo)
    dk = s * (k[1:] - k[:-1])
    d_pair = (dx + dk).astype(np.float64)
    y = x + (s * (k - cm)).astype(np.float64)
    d_ref = y[1:] - y[:-1]
    big = np.maximum(np.abs(dx), np.abs(dk)).astype(np.float32)
    ulp = np.spacing(big).astype(np.float64)
    assert np.all(np.abs(d_pair - d_ref) <= 3.0 * ulp + 2.0 ** -46 * np.abs(x).max())
    # and relative to the size of the differences overall: FP32 accuracy
    assert np.abs(d_pair - d_ref).max() <= 2.0 ** -22 * np.abs(d_ref).max()
