"""Operation counts per facet-trace pair, counted from this package's kernels.

A *pair* is one evaluation of the per-facet raypath physics for one trace
leg; the pair count of a trace is N_ill * (1 + 2 * N_t): the surface leg plus
the inbound and outbound leg of every in-aperture target
(src/CUDA/radar_kernels.cu:714-892).

The fused FP32 kernel (csrc/rp_fast.cu, k_pairs32) evaluates one
(facet, target) combination for both target legs, since the outbound leg is
the inbound one times -1/sqrt(P) in the non-specular mode; so one k_pairs32
evaluation covers two metric pairs.

MUFU (special-function unit) instructions per k_pairs32 evaluation, read off
the source (pair_eval): rsqrt (1/Ttd), the fast division for dT (1), two
rsqrt for the azimuth/inclination projections (2), four sin for the sinc
factors (4), one reciprocal shared by the four sinc quotients (1), exp2 (1)
and sin + cos of the phase (2).
"""

MUFU_PER_EVAL = 12
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
