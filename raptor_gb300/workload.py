"""Algorithmic work of the imaging path, for roofline reporting.

Counted on the oracle's operation-by-operation restatement of the reference
(raptor_port.c compiled with an operation-counting double; pinned by
tests/test_flop_count.py).  Convention: each +, -, *, / and each libm call
(exp, sin, cos, tan, pow, sqrt, log, acos) is one FP64 operation.

  ray set-up       initialize_photon + first r      (metric.c:650-727)
  RK4 step         stepsize + 4 f_geodesic/connection_udd + update + 2 exp(x1)
                   (integrator.c:109-146, 13-41, 274, 283)
  RK2 step         the same with 2 stages            (integrator.c:44-70)
  transfer sample  metric pair + get_fluid_params + pitch angle, plus per
                   frequency k scaling, lower_index, nu_p, j_nu, a_nu, tau, I
                   (radiative_transfer.c:49-119)
"""

FLOP_RAY_SETUP = 138
FLOP_RK4_STEP = 1648
# The survey's hand count of the same algorithm with the connection's
# symmetry used (40 unique symbols, symmetric contraction): 1,260 per RK4
# step and 316 + 63 F per sample.  A lower bar for "achieved", reported
# beside the operation count above.
FLOP_RK4_STEP_SYMMETRIC = 1260
FLOP_SAMPLE_BASE_SYMMETRIC = 316
FLOP_SAMPLE_PER_FREQ_SYMMETRIC = 63
FLOP_RK2_STEP = 814
FLOP_SAMPLE_BASE = 388
FLOP_SAMPLE_PER_FREQ = 109


def image_flops(rays: int, steps: int, samples: int, n_freq: int, rk4: bool = True) -> float:
    """FP64 operations the reference's algorithm spends on one render."""
    step = FLOP_RK4_STEP if rk4 else FLOP_RK2_STEP
    return float(FLOP_RAY_SETUP * rays + step * steps + (FLOP_SAMPLE_BASE + FLOP_SAMPLE_PER_FREQ * n_freq) * samples)


def image_flops_symmetric(steps: int, samples: int, n_freq: int) -> float:
    """The same render's work by the symmetric hand count (RK4)."""
    return float(FLOP_RK4_STEP_SYMMETRIC * steps +
                 (FLOP_SAMPLE_BASE_SYMMETRIC + FLOP_SAMPLE_PER_FREQ_SYMMETRIC * n_freq) * samples)
