"""Operation counts per facet-trace pair, counted from this package's kernels.

A *pair* is one evaluation of the per-facet raypath physics for one trace
leg; the pair count of a trace is N_ill * (1 + 2 * N_t): the surface leg plus
the inbound and outbound leg of every in-aperture target
(src/CUDA/radar_kernels.cu:714-892).

The fused FP32 kernel (csrc/rp_fast.cu, k_pairs32) evaluates one
(facet, target) combination for both target legs, since the outbound leg is
the inbound one times -1/sqrt(P) in the non-specular mode; so one k_pairs32
evaluation covers two metric pairs.

Counts per k_pairs32 evaluation with the polynomial sinc (degree 4, the
large-scene case), read off the source (pair_eval, bin_add fast path):

* FP32 FMA-pipe instructions (FADD/FMUL/FFMA): 82 -- 3+1+1 distance, 1 Ttd,
  2 dT, 6 direction, 3+3 cosines, 6 tangent projections, 3 h^2, 2 (1 - c^2),
  3 squared sinc arguments scale, 4 arguments, 16 polynomials (4 x 4), 3 sinc
  product, 3 exponent, 3 amplitude, 3 phase turns, 1 phase scale, 2 phasor,
  2 bin coordinate, 11 bin split and window update.
* MUFU (special-function) instructions: 6 -- rsqrt (1/Ttd), rcp (dT), rcp
  (1/h^2), ex2, sin and cos of the phase.
"""

FP32_OPS_PER_EVAL = 82
MUFU_PER_EVAL = 6
EVALS_PER_TARGET_PAIR_METRIC = 0.5     # one evaluation covers two metric pairs

# Nominal special-function throughput of a Blackwell SM (results per clock).
MUFU_PER_CLK_PER_SM = 16
FP32_FMA_PER_CLK_PER_SM = 128


def pairs(counts):
    """Metric pair count from (ns, 2) counts [N_ill, N_t]."""
    c = [(int(a), int(b)) for a, b in counts]
    return sum(n * (1 + 2 * t) for n, t in c)


def target_evals(counts):
    """k_pairs32 evaluations: N_ill * N_t per trace."""
    return sum(int(a) * int(b) for a, b in counts)
