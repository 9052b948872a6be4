/*
 * raypath.h -- C ABI of libraypath.so, the GB300 radar-sounder raypath engine.
 *
 * Every function returns an int status: RP_OK (0) or a negative RP_ERR_* code.
 * rp_last_error() returns the text of the calling thread's last error.  No
 * function calls exit(); no function throws across the ABI.
 *
 * Array layouts (all row-major, host pointers unless stated otherwise):
 *   facets   double[12][n]   SoA: x,y,z, nx,ny,nz, ux,uy,uz, vx,vy,vz
 *            (the twelve arrays of loadFacetFile, src/CUDA/file_io.cu:337-362)
 *   targets  double[7][nt]   SoA: x,y,z, nx,ny,nz, ttype
 *            (loadTargetFile, src/CUDA/file_io.cu:365-426)
 *   prisms   double[7][np]   SoA: alpha[Np/m], xmin,ymin,zmin, xmax,ymax,zmax
 *            (loadAttenPrismFile, src/CUDA/file_io.cu:477-517, conductivity
 *            already turned into alpha by rp_prism_alpha)
 *   traces   double[ns][9]   per trace: sx,sy,sz, snx,sny,snz, rst,
 *            grefl_lin, grefr_lin (the per-trace state of the trace loop,
 *            src/CUDA/sim.cu:621-651; the source normal already multiplied by
 *            source_normal_multiplier)
 *   out      float2[ns][nr]  complex64 radargram columns (what
 *            saveSignalToFile writes per trace, src/CUDA/file_io.cu:284-296)
 */
#ifndef RAYPATH_H
#define RAYPATH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    RP_OK = 0,
    RP_ERR_ARG = -1,         /* bad argument or size                           */
    RP_ERR_IO = -2,          /* file missing / unreadable / not a directory    */
    RP_ERR_PARSE = -3,       /* malformed JSON or text record                  */
    RP_ERR_CUDA = -4,        /* CUDA runtime error (text in rp_last_error)     */
    RP_ERR_NOMEM = -5,       /* host or device allocation failed               */
    RP_ERR_UNSUPPORTED = -6, /* mode not implemented by the requested form     */
    RP_ERR_BUDGET = -7,      /* request exceeds the admission memory budget    */
    RP_ERR_TIMEOUT = -8,     /* a bounded wait ran out                         */
    RP_ERR_INTERNAL = -9,    /* invariant violated (bin window overflow, ...)  */
    RP_ERR_CANCELLED = -10   /* the request was cancelled before it started     */
};

#define RP_PENDING 1         /* rp_poll: the request is queued or running      */

/* Simulation form. */
enum {
    RP_FORM_PLAIN_F64 = 0,   /* FP64 restatement of the reference trace loop    */
    RP_FORM_FAST_F32 = 1     /* fused FP32 split-precision form                 */
};

/*
 * Simulation parameters: the JSON keys read by parseSimulationParameters
 * (src/CUDA/file_io.cu:122-249) plus the constants it derives
 * (file_io.cu:168-213).  Fill the inputs, then call rp_params_derive().
 */
typedef struct rp_params {
    /* ---- inputs (JSON keys) ---- */
    double frequency;            /* "frequency"  [Hz]                         */
    double bandwidth;            /* "bandwidth"  [Hz]                         */
    double power;                /* "power"      [W]                          */
    double aperture;             /* "aperture"   [deg]                        */
    double surface_gain;         /* "surface_gain"    [dB]                    */
    double subsurface_gain;      /* "subsurface_gain" [dB]                    */
    double rms_height;           /* "rms_height" [m]                          */
    double buff;                 /* "buff"                                    */
    double eps_1, eps_2;         /* "eps_1", "eps_2"                          */
    double sig_1, sig_2;         /* "sig_1", "sig_2" [S/m]                    */
    double rx_sample_rate;       /* "rx_sample_rate" [Hz]                     */
    double rx_window_m;          /* "rx_window_m" [m]                         */
    double rx_window_offset_m;   /* "rx_window_offset_m" [m] (static rst)     */
    double fs;                   /* "fs" facet size [m]                       */
    double source_normal_multiplier; /* "source_normal_multiplier" (1)        */
    double altitude;             /* "altitude" (0)                            */
    double sx0, sdx, sy, sz;     /* linear source track                       */
    int32_t ns;                  /* "ns"                                      */
    int32_t rerad_funct;         /* "rerad_funct"                             */
    int32_t convolution;         /* "convolution"        (bool)               */
    int32_t convolution_linear;  /* "convolution_linear" (bool)               */
    int32_t specular;            /* "specular"           (bool)               */
    int32_t lossless;            /* "lossless"           (bool)               */
    int32_t incoherent;          /* "incoherent"         (bool, false)        */
    int32_t disable_surface;     /* "disable_surface"    (bool, false)        */
    int32_t debug_surface;       /* "debug_surface"      (bool, false)        */
    int32_t pol;                 /* polarisation: 0 = H (never parsed, 0)     */
    /* ---- derived by rp_params_derive ---- */
    double c;                    /* speed of light                            */
    double lam, k;               /* wavelength, wavenumber                    */
    double rng_res;              /* c / bandwidth                             */
    double grefl_lin, grefr_lin; /* 10^(gain/10)                              */
    double ks;                   /* k * rms_height                            */
    double c_1, c_2;             /* c / sqrt(eps)                             */
    double nu_1, nu_2;           /* 376.7 / sqrt(eps)                         */
    double alpha1, alpha2;       /* attenuation constants [Np/m]              */
    double dr;                   /* rx_window_m / nr                          */
    int32_t nr;                  /* range bins (float expression file_io.cu:212) */
    int32_t reserved;
    /* ---- extension ---- */
    int64_t incoherent_seed;     /* "incoherent_seed" (1): seeds incoherent mode's phases.
                                  * The reference draws them from clock64()
                                  * (randomPhasor, radar_kernels.cu:689-711); here the
                                  * phase of facet i at source (sx, sy, sz) is a
                                  * counter-based hash of (seed, sx, sy, sz, i) --
                                  * reproducible, independent of batching. */
} rp_params;

/* Opaque resident scene (facet store, targets, prisms on the device). */
typedef struct rp_scene rp_scene;

/* Library version string, e.g. "raypath-gb300 1.0". */
const char* rp_version(void);

/* Copy the calling thread's last error text into buf (always terminated). */
int rp_last_error(char* buf, size_t len);

/* Fill the derived fields of p.  Replaces the derivations of
 * parseSimulationParameters, src/CUDA/file_io.cu:167-213. */
int rp_params_derive(rp_params* p);

/* Conductivity [S/m] of an attenuation prism to alpha [Np/m].  Replaces the
 * conversion inside loadAttenPrismFile, src/CUDA/file_io.cu:501-505. */
int rp_prism_alpha(const rp_params* p, double conductivity, double* alpha);

/*
 * Create a resident scene: the facet store is laid out on the device once
 * and reused by every rp_simulate call.  Replaces the facet/target/prism
 * loading and H2D copies of src/CUDA/sim.cu:185-311 and :477-531.
 * device: CUDA device ordinal.
 */
int rp_scene_create(const rp_params* p,
                    const double* facets, int64_t n_facets,
                    const double* targets, int64_t n_targets,
                    const double* prisms, int64_t n_prisms,
                    int device, rp_scene** out);

int rp_scene_destroy(rp_scene* s);

/* Device bytes held by the scene's resident stores. */
int rp_scene_footprint(const rp_scene* s, int64_t* bytes);

/* Device bytes a rp_simulate call of ns traces needs as scratch, per form
 * (an upper bound: every target of the scene taken as in aperture). */
int rp_query_footprint(const rp_scene* s, int64_t ns, int form, int64_t* bytes);

/* The same for a given host trace table (ns x 9): in-aperture target counts
 * from the traces, so the bound is close to what the call reserves. */
int rp_query_footprint_traces(const rp_scene* s, const double* traces, int64_t ns, int form, int64_t* bytes);

/*
 * Simulate ns traces (one radargram column each).  Replaces the trace loop
 * of src/CUDA/sim.cu:615-1008 (one call covers many iterations of it).
 *   traces  host double[ns][9] (see above)
 *   out     float2[ns][nr]; host memory when out_on_device == 0, else device
 *   counts  optional host int64[ns][2]: illuminated facets and in-aperture
 *           targets per trace (the N_ill and N_t of the pair count); may be NULL
 *   stream  cudaStream_t to run on (NULL = the library's own stream)
 * A trace with no illuminated facet yields a zero column (the reference
 * skips writing its file, src/CUDA/sim.cu:693-697; counts report N_ill = 0).
 */
int rp_simulate(rp_scene* s, const double* traces, int64_t ns, int form,
                void* out, int out_on_device, int64_t* counts, void* stream);

/* Same as rp_simulate with the trace table already in device memory
 * (double[ns][9]) -- the resident-input path used for throughput runs. */
int rp_simulate_device(rp_scene* s, const double* d_traces, int64_t ns, int form,
                       void* d_out, int64_t* counts, void* stream);

/* Opaque per-stream scratch.  A scene is read-only while it simulates, so
 * several workspaces (one per concurrent stream or host thread) can run the
 * same resident scene at once; rp_simulate / rp_simulate_device use the
 * scene's own workspace.  New: the reference runs one trace loop at a time
 * (src/CUDA/sim.cu:615). */
typedef struct rp_workspace rp_workspace;

int rp_workspace_create(int device, rp_workspace** out);
int rp_workspace_destroy(rp_workspace* ws);

/* Device bytes currently held by the workspace's scratch. */
int rp_workspace_bytes(const rp_workspace* ws, int64_t* bytes);

/* rp_simulate_device with an explicit workspace (trace table and output in
 * device memory).  Calls sharing a workspace must be ordered on one stream. */
int rp_simulate_ws(rp_scene* s, rp_workspace* ws, const double* d_traces, int64_t ns, int form,
                   void* d_out, int64_t* counts, void* stream);

/* One scene's share of a batch: its trace table and radargram in device
 * memory, counts (ns x 2: N_ill, N_t) in host memory or NULL. */
typedef struct rp_job {
    rp_scene* scene;
    const double* d_traces;   /* ns x 9 float64 */
    int64_t ns;
    void* d_out;              /* ns x nr complex64 */
    int64_t* counts;
} rp_job;

/* Fast form over many scenes at once (uneven facet, target, trace and bin
 * counts, different radar bands): the pair stage of every scene runs in ONE
 * persistent kernel launch (a job table over all scenes' work items), range
 * compression in one launch per bin-count class.  No counterpart in the
 * reference, which runs one scene per process (sim.cu:615-1008); each
 * trace's result is bitwise the one rp_simulate_ws gives, unless the lone
 * call splits its facet parts (rp_split_parts).  Every scene must live on
 * the workspace's device. */
int rp_simulate_batch(const rp_job* jobs, int njobs, rp_workspace* ws, void* stream);

/*
 * CUDA-graph capture of a whole fast-form call.  The reference runs every
 * trace as a host-driven sequence of launches and syncs (sim.cu:615-1008);
 * here one call -- setup, pair stage, compression and tails of every
 * segment, on the caller's stream and the workspace's auxiliary streams --
 * is recorded once and replayed with one graph launch.
 *   rp_graph_create  plans the call from h_traces (host ns x 9, the layout of
 *                    d_traces) with target windows sized by host bounds,
 *                    runs it once eagerly on d_traces / d_out (device
 *                    buffers the graph keeps), then records it.  The graph
 *                    owns its workspace.
 *   rp_graph_launch  replays it on `stream` (NULL: the graph's own stream):
 *                    the results of whatever traces d_traces then holds go
 *                    to d_out.  Replays on one graph must be ordered.
 *   rp_graph_check   after the replay has completed: the status a plain call
 *                    would have returned (a replay whose traces need more
 *                    illuminated-facet or target capacity, or wider target
 *                    windows, than the traces the graph was planned with
 *                    reports RP_ERR_INTERNAL and its output is not valid),
 *                    and the counts (ns x 2: N_ill, N_t) when counts is not
 *                    NULL.
 * Results equal rp_simulate_device's fast form bit for bit.  Fast form,
 * complex64 output only.
 */
typedef struct rp_graph rp_graph;
int rp_graph_create(rp_scene* s, const double* h_traces, const double* d_traces, int64_t ns, void* d_out,
                    rp_graph** out);
/* A whole rp_simulate_batch call recorded as one graph: h_traces[j] is job
 * j's trace table on the host (jobs[j].ns x 9, the layout of
 * jobs[j].d_traces); jobs[j].counts is ignored (rp_graph_check writes the
 * counts of every job in job order, sum of ns x 2).  Every scene must live on
 * one device.  Replays equal direct rp_simulate_batch calls bit for bit. */
int rp_graph_create_batch(const rp_job* jobs, int njobs, const double* const* h_traces, rp_graph** out);
int rp_graph_launch(rp_graph* g, void* stream);
int rp_graph_check(const rp_graph* g, int64_t* counts);
int rp_graph_destroy(rp_graph* g);

/* Pair-kernel autotuner.  With tuning on (the default unless RP_PAIR_CFG
 * fixes a configuration), the first pair launch of each kind (single-scene
 * kernel per sinc degree, or the multi-scene kernel) times the kernel's
 * configurations (facets per step x resident blocks per SM) on a bounded
 * sample of its work items and keeps the fastest for the process.  The
 * configurations give bitwise identical results. */
int rp_autotune(int enable);

/* Split facet parts (on by default).  A fast-form call of one segment whose
 * pair-stage work items (traces x target blocks x 4 facet parts) fill at most
 * half of the pair kernel's resident blocks -- one trace of a small scene, a
 * small serving request -- splits each part's facet range further and folds
 * the split rows back, compensated and in fixed order, before the range
 * compression.  Calls of the same traces give identical results either way
 * to FP32 rounding of each part's compensated sum: a split call can differ
 * from the same trace computed in a larger call or a batch in the last bit
 * (where a part's sum falls within its compensation error of a rounding
 * boundary).  Off: every trace's result is bitwise independent of the call's
 * shape, and small calls leave most of the GPU idle.  Read when a call is
 * planned: a graph keeps the choice it was recorded with. */
int rp_split_parts(int enable);
/* The tuned configuration for (kind, degree), or -1 when not tuned yet.
 * multi: 0 the single-batch kernel (configurations 0-3), 1 multi-segment
 * waves (degree ignored; 0-3 the multi-scene kernel, 4-7 one single-batch
 * kernel per segment in configuration cfg - 4, 8-9 one multi-scene kernel
 * per sinc-degree and frame-kind group), 2 the specular-mode kernel
 * (configurations 0-1). */
int rp_autotune_query(int multi, int degree, int* cfg);

/*
 * Serving: a resident request loop on one device.  No counterpart in the
 * reference, which runs one flyby per process (sim.cu:16-1008).
 *
 * Requests name a resident scene and carry a host trace table (copied at
 * submit) and a caller-owned host output (ns x nr complex64, written before
 * the request completes).  A request is cut into steps of at most
 * step_traces traces (rp_server_configure; by default the whole request is
 * one step).  A request is admitted (becomes active) when its device
 * footprint (the scratch of its largest step plus that step's trace table
 * and output) fits the memory budget next to every active request, and the
 * active limit allows; requests wait in FIFO order.  Each worker call takes
 * the next step of up to max_batch active requests (round robin), then
 * admits queued requests that fit and takes their first step, and runs the
 * fast-form steps it took as one rp_simulate_batch call on its own stream
 * and workspace -- continuous batching at step granularity: requests
 * arriving while others run join at the next call of any worker, short
 * requests finish without waiting for long ones, and the workers' calls
 * overlap on the device.  Plain-form and complex128 steps run one per call.
 * A request's result does not depend on what it was batched or overlapped
 * with.  The queue is internally locked; every function may be called from
 * any thread.
 */
typedef struct rp_server rp_server;

/* Optional executor: run() and footprint() replace the GPU path and
 * rp_query_footprint (the server then makes no CUDA call).  For embedding the
 * queue in front of another engine and for testing the scheduler. */
typedef struct rp_executor {
    int (*run)(void* user, rp_scene* scene, const double* traces, int64_t ns, int form, void* out,
               int64_t* counts);
    int64_t (*footprint)(void* user, rp_scene* scene, int64_t ns, int form);
    void* user;
    /* range bins of a scene (its output row length); may be NULL when
     * requests run whole (no step_traces) */
    int64_t (*bins)(void* user, rp_scene* scene);
} rp_executor;

/* workers >= 1; mem_budget <= 0: 60% of the device's free memory;
 * max_batch >= 1 requests per worker call; ex may be NULL. */
int rp_server_create(int device, int workers, int64_t mem_budget, int max_batch, const rp_executor* ex,
                     rp_server** out);
/* Scheduling options, before the first rp_submit: step_traces > 0 cuts
 * requests into steps of that many traces (0: whole requests); max_active
 * > 0 bounds the requests active at once (0: the budget alone); max_wait_ms
 * > 0 sheds queued requests that waited longer, finishing them with
 * RP_ERR_TIMEOUT (0: no bound).  RP_ERR_ARG after a submit. */
int rp_server_configure(rp_server* srv, int64_t step_traces, int max_active, int max_wait_ms);
/* Drains the queue, then stops the workers. */
int rp_server_destroy(rp_server* srv);
/* Queue a request; *ticket identifies it.  RP_ERR_BUDGET when its footprint
 * alone exceeds the budget (it could never be admitted). */
int rp_submit(rp_server* srv, rp_scene* scene, const double* traces, int64_t ns, int form, void* out,
              int64_t* counts, int64_t* ticket);
/* RP_PENDING while queued or running; once finished, the request's status
 * (RP_OK, an error, RP_ERR_CANCELLED) and the ticket is released.
 * timeout_ms: 0 polls, < 0 waits until the request finishes. */
int rp_poll(rp_server* srv, int64_t ticket, int timeout_ms);
/* Cancel a request that is still queued (RP_ERR_ARG once it is active). */
int rp_cancel(rp_server* srv, int64_t ticket);
/* Wait until nothing is queued or running (timeout_ms < 0: no limit). */
int rp_server_drain(rp_server* srv, int timeout_ms);
/* stats[0..n): completed, failed, rejected, cancelled, p50 ms, p99 ms,
 * mean ms (submit to completion), mean queue wait ms, pairs, pairs/s (first
 * submit to last completion), worker calls, largest batch (steps in one
 * call), footprint in flight (bytes), shed (queue-wait bound), steps run,
 * most requests active at once, most worker calls running at once, p90 ms. */
int rp_server_stats(rp_server* srv, double* stats, int n);

/* Number of kernel launches issued by this thread's last rp_simulate*. */
int rp_last_launch_count(int64_t* launches);

/* Enable (1) / disable (0) per-stage CUDA-event timing of this thread's
 * rp_simulate* calls (events recorded on the launching stream).  Replaces
 * the gettimeofday phase timers of src/CUDA/sim.cu:43-58. */
int rp_set_timing(int enable);

/* Stage times in ms of this thread's last rp_simulate* call:
 *   ms[0] cull + per-facet setup, ms[1] pair kernel, ms[2] per-target range
 *   compression, ms[3] surface compression + final sum; ms[4] (if n > 4) the
 *   number of pair-kernel launches. */
int rp_last_timing(double* ms, int n);

/* ---- the reference's text formats (host only; see rp_io.cu) ---- */

/* Non-blank lines of a text file.  Replaces count_lines,
 * src/CUDA/file_io.cu:314-335. */
int rp_count_records(const char* path, int64_t* n);

/* Facet file "x,y,z:nx,ny,nz:ux,uy,uz:vx,vy,vz" -> double[12][cap].
 * Replaces loadFacetFile, src/CUDA/file_io.cu:337-362. */
int rp_read_facets(const char* path, double* soa, int64_t cap, int64_t* n);

/* Target file, 3/4/6/7 columns (default normal +z, ttype 0) -> double[7][cap].
 * Replaces loadTargetFile, src/CUDA/file_io.cu:365-426. */
int rp_read_targets(const char* path, double* soa, int64_t cap, int64_t* n);

/* Source-path file, 3 or 6 columns -> rows x,y,z,nx,ny,nz.
 * Replaces loadSourceFile, src/CUDA/file_io.cu:429-474. */
int rp_read_sources(const char* path, double* rows, int64_t cap, int64_t* n);

/* Gain-pattern file "surface_dB,subsurface_dB" per line -> rows of 2.
 * Replaces loadGainFile, src/CUDA/file_io.cu:597-624. */
int rp_read_gains(const char* path, double* rows, int64_t cap, int64_t* n);

/* Receive-window starts, exactly ns lines.  Replaces
 * loadRxWindowPositions, src/CUDA/file_io.cu:520-551 (RP_ERR_PARSE instead
 * of exit()). */
int rp_read_rx_window(const char* path, double* out, int64_t ns);

/* Attenuation prisms "sigma,xmin,ymin,zmin,xmax,ymax,zmax" -> double[7][cap]
 * with alpha in row 0.  Replaces loadAttenPrismFile, file_io.cu:477-517. */
int rp_read_prisms(const char* path, const rp_params* p, double* soa, int64_t cap, int64_t* n);

/* Write one trace as "%e %e\n" per bin (re_im: nr complex64 values).
 * Replaces saveSignalToFile, src/CUDA/file_io.cu:284-296. */
int rp_write_trace(const char* path, const float* re_im, int64_t nr);

/* ---- azimuth focusing (src/PYTHON/simple_focusing.py) ------------------
 * The processing step after the simulation.  Radargrams are (Nr range bins,
 * Na traces), row-major, complex64 (in128/out128 = 0) or complex128 (1), in
 * host memory; the work runs on the current device, on stream (a
 * cudaStream_t; NULL = the default stream). */
typedef struct rp_focus_params {
    double rx_window_m, rx_window_offset_m, rx_sample_rate;
    double sin_aperture;    /* sin(aperture in radians), as the caller computes it */
    double spacing;         /* trace spacing (m) */
    double altitude;        /* source altitude (m) */
    double eps_2;           /* subsurface permittivity */
    double lam;             /* wavelength (m) */
    double c1;              /* light speed of the slant-range-to-bin conversion (299792458) */
    double bracket_hi;      /* upper bracket of the refraction angle (radians of 20 degrees) */
} rp_focus_params;

/* focus_rdrgrm (simple_focusing.py:310-404): every pixel of rows
 * [row_lo, row_hi] focused over its range row's synthetic aperture; other
 * rows are zero.  RP_ERR_ARG when a row's refraction angle has no root in
 * [0, bracket_hi] (the reference's brentq raises there). */
int rp_focus_aperture(const rp_focus_params* p, const void* rdr, int64_t nr_bins, int64_t na, int in128,
                      int64_t row_lo, int64_t row_hi, void* out, int out128, void* stream);

/* The per-row geometry of rp_focus_aperture for rows [row0, row0 + nrows):
 * apt[2 r] = apt_smpl, apt[2 r + 1] = apt_hsmpl, and per aperture sample k
 * the range bin rb[r * maxA + k] and matched-filter tap mf[2 (r * maxA + k)]
 * (re, im) -- focus_rdrgrm's return_shifts / return_match_filter. */
int rp_focus_geometry(const rp_focus_params* p, int64_t nr_bins, int64_t row0, int64_t nrows, int maxA, int* apt,
                      int* rb, float* mf);

/* full_focus_at_center (simple_focusing.py:115-185) given its per-trace
 * integer range shifts and matched filter (mf: na complex64 as 2 floats):
 * range-cell-migration correction by rolls and the azimuth matched filter
 * at twice the trace count, cropped to na. */
int rp_focus_center(const void* rdr, int64_t nr_bins, int64_t na, int in128, const int64_t* shifts, const float* mf,
                    void* out, int out128, void* stream);

/* ---- binary stores (the text formats' replacements) -------------------
 * No counterpart in the reference, which parses text with sscanf
 * (loadFacetFile / loadTargetFile, src/CUDA/file_io.cu:337-426) and writes
 * one text file per trace (saveSignalToFile, file_io.cu:284-296).  A store
 * is a 32-byte header (8-byte magic, int64 record count, int64 column or
 * bin count, int64 element kind) followed by the data in the C ABI's own
 * layout: facets "RPFCT01" [12][n] float64 SoA, targets "RPTGT01" [7][n]
 * float64 SoA, radargram "RPRDR01" [ns][nr] complex64 (kind 0) or
 * complex128 (kind 1). */

/* *kind = 0 facet store, 1 target store, 2 radargram, -1 other (text). */
int rp_store_kind(const char* path, int* kind);

/* Write a facet (kind 0) or target (kind 1) store of n records. */
int rp_write_store(const char* path, int kind, const double* soa, int64_t n);

/* Memory-map a facet or target store read-only; *soa stays valid (and may
 * be passed to rp_scene_create) until rp_unmap_store(*handle). */
int rp_map_store(const char* path, int kind, const double** soa, int64_t* n, void** handle);
int rp_unmap_store(void* handle);

/* The whole radargram in one file, trace-major. */
int rp_write_radargram(const char* path, const void* data, int64_t ns, int64_t nr, int complex128);
int rp_radargram_info(const char* path, int64_t* ns, int64_t* nr, int* complex128);
int rp_read_radargram(const char* path, void* data, int64_t ns, int64_t nr, int complex128);

/* The output directory must exist.  Replaces checkDirectoryExists,
 * src/CUDA/file_io.cu:266-281. */
int rp_check_directory(const char* path);

/* Remove s*.txt from dir.  Replaces remove_s_txt_files,
 * src/CUDA/file_io.cu:554-593. */
int rp_clear_traces(const char* dir, int64_t* removed);

/*
 * Surface-only radargram columns with no device allocation at call time.
 * No counterpart in the reference.  For callers that may not allocate
 * device memory once they are running (their device memory budget is fixed
 * up front, e.g. owned by a host application's allocator or a long-running
 * service that must not grow after initialisation): the scene is created
 * beforehand with rp_scene_create, and this call then allocates nothing --
 * its scratch is a fixed 16 MiB array inside the library.
 *   d_traces  device double[ns][9]; d_out device float2[ns][nr]
 *   limits    ns <= 16 traces and nr <= 4096 range bins per call, else
 *             RP_ERR_BUDGET with the limits in rp_last_error()
 *   stream    cudaStream_t to run on (NULL = the scene's own stream, which
 *             is not ordered after work on other streams: pass the stream
 *             that produced d_traces)
 * Accuracy: the incident leg runs in FP64 (the fast form's facet kernel uses
 * FP32 angles), the binning and convolution in the fast form's FP32; the
 * columns agree with rp_simulate_device's fast form for a scene without
 * targets within 1e-6 relative L2, and with the FP64 oracle within 1e-5.
 * Cost: per trace, the facets of the 1024-facet culling tiles that touch the
 * aperture cone are evaluated twice (count and scale, then binning); tiles
 * wholly outside the cone are skipped.
 * Every call shares the one scratch array, and the bins it uses are cleared
 * by each call: calls that overlap on the GPU (different streams, or
 * unordered host threads) race and must not be issued.  Each call looks up
 * the array's device address in the current context (cudaGetSymbolAddress,
 * no allocation); the first call on a device also loads the library's
 * module, so make that first call before any stream capture.
 */
int rp_surface_noalloc(const rp_scene* s, const double* d_traces, int64_t ns, void* d_out,
                       void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RAYPATH_H */
