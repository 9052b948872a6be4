"""Operation counts per facet-trace pair, counted from this package's kernels.

A *pair* is one evaluation of the per-facet raypath physics for one trace
leg; the pair count of a trace is N_ill * (1 + 2 * N_t): the surface leg plus
the inbound and outbound leg of every in-aperture target
(src/CUDA/radar_kernels.cu:714-892).

The fused FP32 kernel (csrc/rp_fast.cu, k_pairs32) evaluates one
(facet, target) combination for both target legs, since the outbound leg is
the inbound one times -1/sqrt(P) in the non-specular mode; so one k_pairs32
evaluation covers two metric pairs.

Counts per k_pairs32 evaluation on the large scene (orthonormal facet
frames, sinc polynomial of degree 3, the fast window path), counted from the
kernel source for the packed two-lane FP32 instructions and measured for the
rest (ncu: executed thread instructions and scalar FFMA/FMUL/FADD over one
launch, divided by the evaluations of that launch); a higher sinc degree
adds 4 FP32 lane operations per degree, general (non-orthonormal) frames
about 10:

* FP32 lane operations: 57.4 -- 52 from packed two-lane instructions (one
  lane per evaluation: anchor distance and Ttd - T0, three direction dot
  products, the four squared sinc arguments, four degree-3 polynomials and
  their product, the attenuation exponent, amplitude, phase, bin coordinate
  and the amplitude-weighted split weights) and 5.4 scalar (the two-bin
  window update from the phase's cosine and sine, and the phase scaling of
  the special-function sine and cosine).
* MUFU (special-function) instructions: 6 -- rsqrt (1/Ttd), rcp (dT), rcp
  (the in-plane split), ex2, sin and cos of the phase.
* All thread instructions: 53.5 -- a packed instruction issues once for two
  evaluations; plus 4 shared-memory record loads and 4 window accesses per
  evaluation, the floor conversion pair, address arithmetic and the loop.
"""

# The reference chain's own cost per leg (its kernels as written: every leg
# recomputes the incident geometry, three facet_G directivities with their
# sinc sines, Snell, Fresnel and the exponentials; geometry_kernels.cu:
# 103-140, 207-350, 410-412, 426-584, radar_kernels.cu:658-892): about 150
# FP32 FMA-class operations and 25 special-function operations per target
# leg, 120 and 20 per surface leg.  This is the algorithmic basis of the
# roofline: the fast form's hoisting (incident terms once per facet and
# trace) and the outbound leg's reuse of the inbound evaluation show up as
# a rate above the FP32 line on this basis.
REF_FMA_PER_TARGET_LEG = 150
REF_SFU_PER_TARGET_LEG = 25
REF_FMA_PER_SURFACE_LEG = 120
REF_SFU_PER_SURFACE_LEG = 20

FP32_OPS_PER_EVAL = 57.4
MUFU_PER_EVAL = 6
INSTR_PER_EVAL = 53.5
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
