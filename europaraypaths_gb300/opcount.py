"""Operation counts per facet-trace pair, counted from this package's kernels.

A *pair* is one evaluation of the per-facet raypath physics for one trace
leg; the pair count of a trace is N_ill * (1 + 2 * N_t): the surface leg plus
the inbound and outbound leg of every in-aperture target
(src/CUDA/radar_kernels.cu:714-892).

The fused FP32 kernel (csrc/rp_fast.cu, k_pairs32) evaluates one
(facet, target) combination for both target legs, since the outbound leg is
the inbound one times -1/sqrt(P) in the non-specular mode; so one k_pairs32
evaluation covers two metric pairs.

Counts per k_pairs32 evaluation on the large scene (sinc polynomial of
degree 3, the fast window path), measured from the kernel's executed
instruction mix (ncu sass__inst_executed_per_opcode over one launch, divided
by the evaluations of that launch); a higher sinc degree adds 4 FFMA per
degree:

* FP32-pipe instructions: 72 -- 34 FFMA, 26 FMUL, 10 FADD, 2 compare and
  select.  The terms: distance and Ttd - T0 from the anchor, the four
  direction dot products, 1 - cos^2 of both angles, the in-plane sinc split,
  four degree-3 polynomials and their product, the attenuation exponent,
  amplitude, phase and its scaling, phasor, bin coordinate, and the two-bin
  window update.
* MUFU (special-function) instructions: 7 -- rsqrt (1/Ttd), rcp (dT), rcp
  (1/Ttd^2), rcp (1/h^2), ex2, sin and cos of the phase.
* All instructions (the issue rate that bounds the kernel): 97.5 -- the
  above plus 6 shared-memory accesses (record and window), the floor
  conversion pair, address arithmetic and the loop.
"""

FP32_OPS_PER_EVAL = 72
MUFU_PER_EVAL = 7
INSTR_PER_EVAL = 97.5
EVALS_PER_TARGET_PAIR_METRIC = 0.5     # one evaluation covers two metric pairs

# Nominal special-function throughput of a Blackwell SM (results per clock).
MUFU_PER_CLK_PER_SM = 16
FP32_FMA_PER_CLK_PER_SM = 128
ISSUE_PER_CLK_PER_SM = 128      # 4 schedulers x one 32-thread instruction per clock


def pairs(counts):
    """Metric pair count from (ns, 2) counts [N_ill, N_t]."""
    c = [(int(a), int(b)) for a, b in counts]
    return sum(n * (1 + 2 * t) for n, t in c)


def target_evals(counts):
    """k_pairs32 evaluations: N_ill * N_t per trace."""
    return sum(int(a) * int(b) for a, b in counts)
