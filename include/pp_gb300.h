/*
 * pp_gb300.h -- C ABI of the GB300 (sm_103a) photon-transport library.
 *
 * This is the drop-in seam for PhotonPropagation.jl's photon-transport hot path.
 * Julia reaches it through `ccall`; Python through ctypes.  Every function
 * returns an int status (pp_status); a message for the last failure on the
 * calling thread is available from pp_last_error().
 *
 * Reference interfaces replaced (PhotonPropagation.jl v0.9.3, paths inside
 * that project):
 *   run_photon_prop_no_local_cache!   src/photon_prop_cuda.jl:889-959
 *   cuda_propagate_photons!           src/photon_prop_cuda.jl:429-549
 *   make_hit_buffers                  src/photon_prop_cuda.jl:878-886
 *   PhotonPropOOMException            src/photon_prop_cuda.jl:40, :937-939
 *   PhotonPropSetup (device tables)   src/photon_propagation_setup.jl:18-25
 *   make_cuda_spectral_dist           src/spectrum.jl:75-83
 *
 * Conventions
 *   - 0 = success; 1 = hit buffer overflow (the Julia shim throws
 *     PhotonPropOOMException, as src/photon_prop_cuda.jl:937-939 does);
 *     negative = invalid argument / CUDA error / bounded device wait gave up.
 *   - A context owns one device, one internal stream and its device tables.
 *     Calls on one context are not re-entrant; separate contexts may be used
 *     from separate threads.
 *   - pp_propagate is synchronous with respect to the caller (like the
 *     reference's CUDA.@sync launch, src/photon_prop_cuda.jl:933).  pp_launch
 *     and pp_launch_graph are asynchronous on the caller's stream.
 *   - No function ever falls back to a CPU implementation: without a usable
 *     CUDA device they return PP_ERR_NO_DEVICE.
 */
#ifndef PP_GB300_H
#define PP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define PP_API __declspec(dllexport)
#else
#define PP_API __attribute__((visibility("default")))
#endif

#define PP_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define PP_OK 0
#define PP_ERR_OVERFLOW 1    /* hit buffer full: PhotonPropOOMException      */
#define PP_ERR_INVALID (-1)  /* bad argument                                 */
#define PP_ERR_CUDA (-2)     /* CUDA runtime error (message in last_error)    */
#define PP_ERR_TIMEOUT (-3)  /* a bounded device-side wait gave up            */
#define PP_ERR_NOT_READY (-4)/* medium / spectrum / targets / sources missing */
#define PP_ERR_NO_DEVICE (-5)/* no CUDA device                                */

/* ---- device-side error flag bits (pp_counters.err_flags) ---------------- */
#define PP_FLAG_OVERFLOW 1u  /* a hit did not fit into the buffer            */
#define PP_FLAG_TIMEOUT 2u   /* a TMA staging wait hit its iteration limit    */

/* ---- emitter kinds (src/lightyield.jl:437-873, init functions
 *      src/photon_prop_cuda.jl:158-276) ----------------------------------- */
#define PP_SRC_POINTLIKE_ISOTROPIC 0        /* lightyield.jl:549, prop:158  */
#define PP_SRC_EXTENDED_CHERENKOV 1         /* lightyield.jl:616, prop:211  */
#define PP_SRC_EXTENDED_CHERENKOV_NOSMEAR 2 /* lightyield.jl:670, prop:225  */
#define PP_SRC_POINTLIKE_CHERENKOV 3        /* prop:254                     */
#define PP_SRC_CHERENKOV_TRACK 4            /* prop:265                     */
#define PP_SRC_POINTLIKE_TIME_RANGE 5       /* lightyield.jl:592, prop:165  */
#define PP_SRC_COLLIMATED_ISOTROPIC 6       /* lightyield.jl:570, prop:186  */
#define PP_SRC_PENCIL 7                     /* lightyield.jl:527, prop:197  */
#define PP_SRC_AXICONE 8                    /* lightyield.jl:503, prop:173  */
#define PP_SRC_KIND_COUNT 9

/* One photon source (96 bytes).  Fields not used by a kind are ignored.
 * The source emits photons first_photon .. first_photon + n - 1 (n after
 * scaling); photon i always draws the same random numbers, so a source can be
 * split into photon ranges (shards, replays) with identical results. */
typedef struct pp_source {
  int32_t kind;           /* PP_SRC_*                                         */
  int32_t smear_table;    /* Cherenkov kinds: track-smear table (0 = first)   */
  int64_t photons;        /* PhotonSource.photons (Int64)                     */
  float position[3];      /* m                                                */
  float time;             /* ns; time_range[1] for POINTLIKE_TIME_RANGE       */
  float direction[3];     /* unit axis (Cherenkov, pencil, axicone)           */
  float time_end;         /* ns; time_range[2] for POINTLIKE_TIME_RANGE       */
  float long_a;           /* LongitudinalParameterisation.a                   */
  float long_b;           /* LongitudinalParameterisation.b                   */
  float long_lrad;        /* LongitudinalParameterisation.lrad (m)            */
  float length;           /* CherenkovTrackEmitter.length (m)                 */
  float angle;            /* AxiconeEmitter.angle (rad)                       */
  float beam_divergence;  /* Axicone / Pencil beam_divergence (rad)           */
  float cut_angle_cos;    /* CollimatedIsotropicEmitter.cut_angle_cos         */
  float reserved1;
  int64_t first_photon;   /* index of the first photon (0 for a whole source) */
  int64_t reserved2;
} pp_source;

/* Spherical{Float32} target (NeutrinoTelescopeBase): 16 bytes. */
typedef struct pp_sphere {
  float position[3];
  float radius;
} pp_sphere;

/* Medium as tables on a uniform wavelength grid, plus the MixedHGES phase
 * function (CascadiaMediumProperties, src/water_properties.jl:43-100;
 * SimpleMediumProperties, src/simple_medium.jl:1-15).  The Julia shim fills
 * the tables with the reference's own scattering_length / group_velocity /
 * absorption_length / phase_refractive_index. */
#define PP_PHASE_HG_ES 0  /* MixedHGES: HG(g) or Einstein-Smoluchowski(b) (water)       */
#define PP_PHASE_HG_SL 1  /* HG(g) or simplified Liu(g), cos = 2 u^((1-g)/(1+g)) - 1
                             (mixed_hg_sl_scattering_func_ppc, deep ice)              */
typedef struct pp_medium {
  float wl_min;                       /* nm of knot 0                        */
  float wl_step;                      /* nm between knots (> 0)              */
  int32_t n_knots;                    /* >= 2                                */
  int32_t phase_kind;                 /* PP_PHASE_*                          */
  const float* scattering_length;     /* m    [n_knots]                      */
  const float* group_velocity;        /* m/ns [n_knots]                      */
  const float* absorption_length;     /* m    [n_knots]                      */
  const float* phase_refractive_index;/*      [n_knots]                      */
  float hg_g;                         /* Henyey-Greenstein mean cosine       */
  float es_b;                         /* Einstein-Smoluchowski b (HG_ES)     */
  float hg_weight;                    /* P(HG) in the mixture; 1 = pure HG   */
  float reserved1;
} pp_medium;

/* Launch tuning (chosen by pp_autotune or set by the caller). */
typedef struct pp_tuning {
  int32_t block_threads;      /* CTA size, multiple of 32, 64..1024          */
  int32_t photons_per_thread; /* photons each lane takes per queued chunk    */
  int32_t ctas_per_sm;        /* 0 = occupancy maximum                       */
  int32_t precise_math;       /* 1 = IEEE libm functions (replay checks)     */
  float cell_size;            /* target-grid cell edge (m); 0 = automatic    */
  int32_t grid_in_global;     /* 1 = read the grid from global memory        */
  float safety_cell;          /* safety-field cell edge (m); 0 = automatic   */
  int32_t target_loop;        /* 1 = no culling: every sphere is tested at    */
                              /* every step in index order, the reference's   */
                              /* own loop (src/photon_prop_cuda.jl:497-506);  */
                              /* same hits, for comparisons                   */
} pp_tuning;

/* One hit as written by the kernel into device memory: 80 bytes, 16-byte
 * aligned, stored with vectorised 16-byte stores.  Fields follow PhotonHit
 * (src/photon_prop_cuda.jl:407-416) plus the absorption weight that the
 * reference computes on the host (src/processing.jl:32-44). */
typedef struct pp_hit_record {
  /* the first 32 bytes hold what the detection step reads (one sector) */
  float position[3];
  float wavelength;
  float direction[3];
  int32_t module_index;       /* 1-based index into the target list            */
  float dist_travelled;
  float initial_direction[3];
  float abs_weight;           /* exp(-dist_travelled / absorption_length)     */
  int32_t n_steps;            /* step (1-based) at which the photon hit        */
  int32_t source_index;       /* 0-based index into the source list            */
  int32_t reserved;
  double time;                /* ns (FP64 accumulator)                         */
  int64_t photon_index;       /* index of the photon within its source         */
} pp_hit_record;

/* Device-side counters of one launch (zeroed by pp_launch / pp_launch_graph). */
typedef struct pp_counters {
  uint64_t n_hits;        /* hit slots claimed (> capacity on overflow)      */
  uint64_t n_ph_sim;      /* photons fully simulated                          */
  uint64_t photon_steps;  /* scattering steps taken, all photons              */
  uint64_t work_next;     /* head of the device work queue                    */
  uint32_t err_flags;     /* PP_FLAG_*                                        */
  uint32_t reserved[3];
} pp_counters;

/* Hit table as columns (structure of arrays), host or device memory, each
 * column caller-allocated with room for `capacity` rows.  Vector columns are
 * row-major [n][3].  NULL columns are skipped. */
typedef struct pp_hits {
  float* position;
  float* direction;
  float* initial_direction;
  float* wavelength;
  double* time;
  float* dist_travelled;
  float* abs_weight;
  int32_t* module_index;
  int32_t* n_steps;
  int32_t* source_index;
  int64_t* photon_index;
} pp_hits;

typedef struct pp_ctx pp_ctx;

/* ---- library ------------------------------------------------------------ */

/* ABI version (PP_ABI_VERSION).  No reference counterpart. */
PP_API int pp_version(void);

/* Copy the calling thread's last error message into buf (always
 * NUL-terminated); returns the full message length. */
PP_API int pp_last_error(char* buf, int32_t len);

/* ---- context ------------------------------------------------------------ */

/* Create a context on `device`.  Replaces the implicit CUDA.jl device state
 * used by run_photon_prop_no_local_cache! (src/photon_prop_cuda.jl:889-912). */
PP_API int pp_create(pp_ctx** out, int32_t device);
PP_API int pp_destroy(pp_ctx* ctx);

/* Medium tables (the per-wavelength evaluations the kernel performs with
 * scattering_length / group_velocity at src/photon_prop_cuda.jl:480-482 and
 * the host absorption weight at src/processing.jl:38-39). */
PP_API int pp_set_medium(pp_ctx* ctx, const pp_medium* medium);

/* Tabulated inverse CDF of the wavelength spectrum, n knots at u=i/(n-1)
 * (make_cuda_spectral_dist, src/spectrum.jl:75-83).  Sampled like the
 * reference's 1-D linear-filtered texture with normalised coordinates. */
PP_API int pp_set_spectrum(pp_ctx* ctx, const float* inv_cdf_knots, int32_t n);

/* Monochromatic spectrum (Monochromatic, src/spectrum.jl:66-72). */
PP_API int pp_set_monochromatic(pp_ctx* ctx, float wavelength_nm);

/* Quantile table of cos(theta) of the Cherenkov track direction about the
 * emitter axis, n knots at u=i/(n-1) (sample_cherenkov_track_direction,
 * called at src/photon_prop_cuda.jl:89).  Needed by Cherenkov emitters. */
PP_API int pp_set_track_smear(pp_ctx* ctx, const float* cos_theta_quantiles, int32_t n);

/* n_tables such tables of n knots each, table t at cos_theta_quantiles[t * n];
 * a Cherenkov source draws from table pp_source.smear_table.  One table per
 * distinct Beta(a, b) of ExtendedCherenkovEmitterCustomSmear (track cos theta
 * = 2 Beta(a, b) - 1, src/photon_prop_cuda.jl:134-154, src/lightyield.jl:
 * 725-769).  pp_set_track_smear is the one-table form. */
PP_API int pp_set_track_smear_tables(pp_ctx* ctx, const float* cos_theta_quantiles, int32_t n,
                                     int32_t n_tables);

/* Upload spherical targets and build the uniform culling grid on the device.
 * cell_size <= 0 picks a size automatically.  Replaces CuVector(targets)
 * (src/photon_prop_cuda.jl:910-912). */
PP_API int pp_set_targets(pp_ctx* ctx, const pp_sphere* targets, int32_t n, float cell_size);

/* Upload the source list and build the device work queue.  Photon count of
 * source i is floor(Float32(photons) * photon_scaling), computed in FP32 as the
 * reference does (src/photon_prop_cuda.jl:456). */
PP_API int pp_set_sources(pp_ctx* ctx, const pp_source* sources, int32_t n, float photon_scaling);

PP_API int pp_set_tuning(pp_ctx* ctx, const pp_tuning* tuning);
PP_API int pp_get_tuning(const pp_ctx* ctx, pp_tuning* tuning);

/* Total photons of the uploaded sources after scaling. */
PP_API int pp_total_photons(const pp_ctx* ctx, int64_t* total);

/* ---- propagation ---------------------------------------------------------- */

/* Targets of any shape (src/photon_prop_cuda.jl:345-404): spheres, and the
 * horizontal (normal e_z) rectangle and disc of the reference's Rectangular
 * and Circular shapes.  With any non-spherical target the kernel tests every
 * target at every step in index order, as the reference does (no culling
 * grid); a list of spheres only takes the culled path of pp_set_targets.
 *
 * DetectorLines (the kernel variant of src/photon_prop_cuda.jl:552-694): the
 * list is L groups of one PP_TARGET_LINE record (position[0..1] = the line's
 * x, y; radius = its 2-D radius; reserved = N, the same for every line)
 * followed by its N module records (any shape).  At each step the lines are
 * tested in order with the 2-D ray-circle test of the step's (x, y) start
 * and its unnormalised (x, y) direction over the 3-D step length; the first
 * crossed line ends the search whether or not one of its modules is hit, and
 * a hit on module t (1-based) of line l (1-based) reports module index
 * t + N * l, all as the reference computes them.  N * (L + 1) <= 65535. */
#define PP_TARGET_SPHERE 0
#define PP_TARGET_RECTANGLE 1
#define PP_TARGET_DISC 2
#define PP_TARGET_LINE 3
typedef struct pp_target {
  float position[3];
  float radius;      /* sphere, disc, line */
  float length_x;    /* rectangle */
  float length_y;    /* rectangle */
  int32_t kind;      /* PP_TARGET_* */
  int32_t reserved;  /* line: modules per line */
} pp_target;
PP_API int pp_set_shaped_targets(pp_ctx* ctx, const pp_target* t, int32_t n);

/* Asynchronous launch on `stream` (cudaStream_t; NULL = legacy default
 * stream): zeroes *d_counters, runs the persistent propagation kernel over
 * every uploaded source, writes hits into d_hits (device memory, capacity
 * records).  The pp_set_* calls of a context first wait for its launches
 * (pp_launch, pp_launch_histogram, pp_launch_graph) still running, since
 * they overwrite the device inputs those launches read; so a caller may
 * upload the next batch of sources right after a launch.  The device-resident form of cuda_propagate_photons! launched
 * once per source (src/photon_prop_cuda.jl:927-943): here one launch covers
 * all sources through a device work queue. */
PP_API int pp_launch(pp_ctx* ctx, int64_t seed, int32_t n_steps, pp_hit_record* d_hits,
                     int64_t capacity, pp_counters* d_counters, void* stream);

/* Histogram form of pp_launch for photon-table generation: no hit records;
 * every hit of source s adds its absorption weight to d_hist[s*(n_bins+1)]
 * (expected hits) and to bin 1 + b, b the bin of
 * log10(t - d_tgeo[s] + t_offset) on n_bins uniform bins over [log_lo, log_hi)
 * (clamped into the edge bins).  d_tgeo: per-source geometric time (ns),
 * device memory.  Replaces the hit-table -> per-PMT counts -> residual-time
 * histogram pipeline of the reference's table scripts
 * (scripts/photon_tables/photon_tables_photons.jl:33-151,
 * src/calc.jl calc_time_residual!). */
PP_API int pp_launch_histogram(pp_ctx* ctx, int64_t seed, int32_t n_steps, const float* d_tgeo,
                               float* d_hist, int32_t n_bins, float t_offset, float log_lo,
                               float log_hi, pp_counters* d_counters, void* stream);

/* Same work as pp_launch, replayed from a CUDA graph (memset + kernel)
 * captured on first use for these arguments. */
PP_API int pp_launch_graph(pp_ctx* ctx, int64_t seed, int32_t n_steps, pp_hit_record* d_hits,
                           int64_t capacity, pp_counters* d_counters, void* stream);

/* Synchronous drop-in for run_photon_prop_no_local_cache!
 * (src/photon_prop_cuda.jl:889-959): uploads `sources`, propagates, and
 * copies only the n_hits rows (not the whole buffer) into `out` (host or
 * device columns with room for `capacity` rows; out = NULL copies nothing,
 * see pp_fetch_hits).  Returns PP_ERR_OVERFLOW when more than `capacity` hits
 * occurred (*n_hits then holds the number of hits).  The device hit buffer is
 * owned by the context and holds min(capacity, photons) records (a photon hits
 * at most once). */
PP_API int pp_propagate(pp_ctx* ctx, const pp_source* sources, int32_t n_src, int64_t seed,
                        int32_t n_steps, float photon_scaling, const pp_hits* out,
                        int64_t capacity, int64_t* n_hits, int64_t* n_ph_sim);

/* Copy the first n hits of the last pp_propagate on this context into `out`
 * (host or device columns with room for n rows).  With pp_propagate(out=NULL)
 * this lets a caller size its output after the hit count is known, copying
 * only n_hits rows (the reference copies the whole buffer,
 * src/photon_prop_cuda.jl:950-954). */
PP_API int pp_fetch_hits(pp_ctx* ctx, const pp_hits* out, int64_t n);

/* Free and total memory of `device` in bytes (CUDA.totalmem as used by
 * make_hit_buffers, src/photon_prop_cuda.jl:878-880). */
PP_API int pp_device_memory(int32_t device, int64_t* free_bytes, int64_t* total_bytes);

/* Size of the device array that pp_propagate_static takes its scratch from. */
#define PP_STATIC_SCRATCH_BYTES (8u * 1024u * 1024u)

/* Propagation that allocates no device memory.  No counterpart in the
 * reference: it is for callers that cannot call cudaMalloc -- code running
 * while another framework's pooling allocator owns the device memory, and
 * services that fix their memory use at start-up.  Inputs are host arrays (medium tables, spectrum knots or
 * a monochromatic wavelength, one track table (sources' smear_table 0),
 * spherical targets, sources); hits go to the
 * caller's device buffer d_hits (16-byte aligned, `capacity` records) and the
 * launch's counters to the host struct *counters.  All scratch (device copies
 * of the inputs, culling grid, safety field, work queue, counters) comes from
 * one static device array of PP_STATIC_SCRATCH_BYTES (8 MiB), which every GPU
 * that loads this library holds until exit; inputs needing more are rejected
 * with PP_ERR_INVALID.  The first call on a device looks up the array's
 * address: make it before any stream capture.  Calls share the array, so calls
 * that overlap on the GPU race.  Runs on the current device, synchronously on
 * `stream`: it copies the inputs from host memory, reads counters back and
 * synchronises the stream, so a call cannot be recorded by stream capture.
 * Returns PP_ERR_OVERFLOW when more than `capacity` hits occur. */
PP_API int pp_propagate_static(const pp_medium* medium, const float* spectrum_knots,
                               int32_t n_spectrum, float mono_wavelength,
                               const float* track_quantiles, int32_t n_track,
                               const pp_sphere* targets, int32_t n_targets, float cell_size,
                               const pp_source* sources, int32_t n_src, int64_t seed,
                               int32_t n_steps, float photon_scaling, pp_hit_record* d_hits,
                               int64_t capacity, pp_counters* counters, void* stream);

/* Scatter n device hit records into device columns (structure of arrays). */
PP_API int pp_hits_to_columns(const pp_hit_record* d_records, int64_t n, const pp_hits* d_out,
                              void* stream);

/* Time candidate tunings on a sample of the uploaded sources and keep the
 * fastest (block size, photons per thread, grid cell size).  No reference
 * counterpart (the reference uses CUDA.launch_configuration,
 * src/photon_prop_cuda.jl:914-921). */
PP_API int pp_autotune(pp_ctx* ctx, int64_t seed, int32_t n_steps, int64_t sample_photons,
                       pp_tuning* best, double* best_photons_per_s);

/* ---- learned surrogate (no reference counterpart: the reference evaluates an
 *      external PhotonSurrogateModel, examples/validation.jl:455,673-676) ---- */

/* A small MLP (n_in -> n_layers x hidden SiLU -> 1 + n_bins) mapping
 * source-module geometry to log expected hits and arrival-time logits,
 * trained with BF16 tcgen05 kernels (FP32 accumulate, Poisson + multinomial
 * NLL, Adam).  Parameters are packed FP32: for each layer W (rows x cols,
 * padded, row-major) then b (rows), see pp_mlp_layout. */
typedef struct pp_mlp pp_mlp;
PP_API int pp_mlp_create(pp_mlp** out, int32_t device, int32_t n_in, int32_t hidden,
                         int32_t n_layers, int32_t n_bins, int32_t max_batch, uint64_t seed);
PP_API int pp_mlp_destroy(pp_mlp* mlp);
PP_API int pp_mlp_num_params(const pp_mlp* mlp, int64_t* n);
PP_API int pp_mlp_layout(const pp_mlp* mlp, int32_t layer, int64_t* off_w, int64_t* off_b,
                         int32_t* rows, int32_t* cols);
PP_API int pp_mlp_get_params(const pp_mlp* mlp, float* host, int64_t n);
PP_API int pp_mlp_set_params(pp_mlp* mlp, const float* host, int64_t n);
/* Training-graph forward: d_x (B x n_in, FP32, device) -> d_out (B x padded
 * outputs, FP32, device): column 0 log expected count, 1..n_bins time logits. */
PP_API int pp_mlp_forward(pp_mlp* mlp, const float* d_x, int32_t B, float* d_out, void* stream);
/* Loss and parameter gradients (no update); host outputs may be NULL. */
PP_API int pp_mlp_loss_grad(pp_mlp* mlp, const float* d_x, const float* d_count,
                            const float* d_hist, int32_t B, float* host_grad, float* host_loss,
                            void* stream);
/* One Adam step (forward, backward, update), asynchronous on `stream`. */
PP_API int pp_mlp_train_step(pp_mlp* mlp, const float* d_x, const float* d_count,
                             const float* d_hist, int32_t B, float lr, void* stream);
/* n_steps Adam steps run by the library: each draws a batch of B rows
 * uniformly, with replacement, from the n_rows training rows in device memory
 * (d_x n_rows x n_in, d_count n_rows, d_hist n_rows x n_bins; row i of the
 * batch of Adam step t is Philox4x32-10(i, t, tag; key = seed) scaled to
 * n_rows), and takes a step of size lr1 + (lr0 - lr1) (1 + cos(pi s / (total - 1))) / 2,
 * s = t - step0 the step's index in a cosine schedule that began at Adam step
 * step0.  One step is captured once as a CUDA graph (for these arguments) and
 * replayed, so n_steps calls cost n_steps graph launches; batches and step
 * sizes depend only on the global step index, so K1 then K2 steps equal
 * K1 + K2 steps in one call.  Asynchronous on `stream`. */
PP_API int pp_mlp_train_steps(pp_mlp* mlp, const float* d_x, const float* d_count,
                              const float* d_hist, int64_t n_rows, int32_t B, int32_t n_steps,
                              int64_t step0, int64_t total, float lr0, float lr1, uint64_t seed,
                              void* stream);
/* Adam steps taken so far. */
PP_API int pp_mlp_step_count(const pp_mlp* mlp, int64_t* steps);
PP_API int pp_mlp_last_loss(pp_mlp* mlp, float* host_loss);
/* Adam moments (n = pp_mlp_num_params floats each; NULL skips one on get)
 * and step count, for training checkpoints. */
PP_API int pp_mlp_get_adam(const pp_mlp* mlp, float* host_m, float* host_v, int64_t n,
                           int64_t* step);
PP_API int pp_mlp_set_adam(pp_mlp* mlp, const float* host_m, const float* host_v, int64_t n,
                           int64_t step);
/* Fused inference (one tcgen05 kernel; activations stay in shared memory):
 * d_x (n x n_in, FP32, device) -> d_expect[n] = exp(min(log-count, 30)) and,
 * when d_pdf is not NULL, d_pdf (n x n_bins) = softmax of the time logits.
 * Computed with BF16 weights and activations and FP32 accumulation, the
 * rounding points of the training forward pass; BF16 keeps FP32's exponent
 * range, so a finite network cannot saturate.  The Python layer bounds the
 * hidden activations over an input box by interval arithmetic
 * (surrogate.activation_bound) and fails a serving batch whose network could
 * overflow BF16.
 * Asynchronous on `stream`; n is not limited by max_batch.  Timeouts of the
 * kernel's waits set a device flag that pp_mlp_check reports. */
PP_API int pp_mlp_infer(pp_mlp* mlp, const float* d_x, int64_t n, float* d_expect, float* d_pdf,
                        void* stream);
/* Diagnostic of the inference kernel's bounded waits (no reference
 * counterpart): pp_mlp_infer with every wait bounded to wait_ns
 * (1e3..2e9 ns) and the first weight chunk's barrier armed but its copy not
 * issued, so that the waits on it run out with nothing of theirs in flight;
 * the kernel winds down (its own copies awaited, tensor memory freed) and the
 * call returns PP_ERR_TIMEOUT (flag cleared) when the bounds work.  Waits for
 * `stream`. */
PP_API int pp_mlp_debug_infer_timeout(pp_mlp* mlp, const float* d_x, int64_t n, float* d_expect,
                                      int64_t wait_ns, void* stream);
/* Synchronises `stream`; PP_ERR_TIMEOUT (and clears the flag) if a
 * tensor-core wait of an earlier MLP kernel gave up. */
PP_API int pp_mlp_check(pp_mlp* mlp, void* stream);
/* One tcgen05 GEMM (test hook): C = A * B^T, BF16 in, FP32 out (k_split > 0:
 * C += over K slices). */
PP_API int pp_mlp_gemm_test(const void* d_a, int64_t lda, int32_t a_trans, const void* d_b,
                            int64_t ldb, int32_t b_trans, int32_t M, int32_t N, int32_t K,
                            int32_t k_split, float* d_c, int64_t ldc, void* stream);

/* ---- photon hits -> PMT hits (make_hits_from_photons, calc_pe_weight!) ---- */

#define PP_PMT_HOMOGENEOUS 0   /* detected with probability active_area / (4 pi r^2) */
#define PP_PMT_POM 1           /* 16-PMT optical module, POMAcceptance               */
#define PP_PMT_DOM 2           /* single-PMT DOM, DOMAcceptance                      */
#define PP_PMT_MULTIPMT 3      /* SphericalMultiPMTTarget (generic multi-PMT module) */
#define PP_POM_MAX_KNOTS 128
#define PP_DOM_MAX_POLY 16
#define PP_MULTIPMT_MAX_PMTS 32

/* One module as the detection step sees it (target i of the propagation is
 * module_index i + 1 of its hit records). */
typedef struct pp_pmt_target {
  float position[3];
  float radius;
  int32_t kind;            /* PP_PMT_*                                        */
  float active_area;       /* m^2, PP_PMT_HOMOGENEOUS                          */
} pp_pmt_target;

/* The POM model (src/pom.jl:16-34,63-160): PMT directions in the detector
 * frame (the reference's pmt_coordinates after the module orientation),
 * PMT groups (1 or 2), per-group Rayleigh widths of the angular acceptance and
 * total acceptance vs wavelength (assets/pmt_acc.hd5), and the relative
 * quantum efficiency vs wavelength (assets/PMTAcc.csv).  Knots ascending. */
typedef struct pp_pom_model {
  int32_t n_acc;
  int32_t n_qe;
  float acc_wavelength[PP_POM_MAX_KNOTS];
  float acc_group1[PP_POM_MAX_KNOTS];
  float acc_group2[PP_POM_MAX_KNOTS];
  float sigma_group1;
  float sigma_group2;
  float qe_wavelength[PP_POM_MAX_KNOTS];
  float qe[PP_POM_MAX_KNOTS];
  float pmt_dir[16][3];
  int32_t pmt_group[16];
} pp_pom_model;

/* The DOM model (src/dom.jl:8-26,96-134): an angular acceptance polynomial in
 * the cosine of the photon direction's zenith in the module frame (coefficients
 * in ascending powers, its maximum `polymax`) and a wavelength acceptance
 * (assets/icecube_wl_acc.csv divided by the DOM's cross-section).
 * zenith_axis = the third column of the module orientation, so that
 * cos zenith = zenith_axis . direction = (inv(orientation) * direction)[3].
 * apply_wl_acceptance = 0 skips the wavelength test (make_hits_from_photons
 * with apply_wl_acc = false, src/processing.jl:126-128). */
typedef struct pp_dom_model {
  int32_t n_poly;
  int32_t n_wl;
  float poly[PP_DOM_MAX_POLY];
  float polymax;
  float zenith_axis[3];
  int32_t apply_wl_acceptance;
  float wl[PP_POM_MAX_KNOTS];
  float wl_acc[PP_POM_MAX_KNOTS];
} pp_dom_model;

/* The generic multi-PMT module (src/detection.jl:90-131,
 * src/generic_multipmt.jl): n_pmt PMTs of area pmt_area; the PMT axes in the
 * module frame (the projected-area hit probability uses them unrotated, as the
 * reference does) and after the module orientation (the PMT choice); the
 * quantum efficiency vs wavelength (assets/R6091_relqe.csv, QE / 100). */
typedef struct pp_multipmt_model {
  int32_t n_pmt;
  int32_t n_qe;
  float pmt_area;
  float pmt_dir_module[PP_MULTIPMT_MAX_PMTS][3];
  float pmt_dir[PP_MULTIPMT_MAX_PMTS][3];
  float qe_wavelength[PP_POM_MAX_KNOTS];
  float qe[PP_POM_MAX_KNOTS];
} pp_multipmt_model;

/* The detection models of one call; a model may be NULL when no target has
 * its kind. */
typedef struct pp_detection_models {
  const pp_pom_model* pom;
  const pp_dom_model* dom;
  const pp_multipmt_model* multipmt;
} pp_detection_models;

/* Detection of n photon hits (device hit records as the propagation writes
 * them): d_pmt_id[i] = 1-based PMT index, 0 = not detected; d_qe_weight[i]
 * (may be NULL) = relative quantum efficiency at the hit's wavelength (the
 * factor calc_pe_weight! multiplies into total_weight; 1 for homogeneous
 * modules).  Replaces the per-module host loops of make_hits_from_photons
 * (src/processing.jl:88-139) with check_pmt_hit (src/pom.jl:246-305,
 * src/detection.jl:57-84) and calc_pe_weight! (src/processing.jl:179-205);
 * random numbers from a Philox stream keyed on `seed` (the reference draws
 * from Julia's global RNG).  Asynchronous on `stream`; `targets` and `pom`
 * are host structs copied before the call returns. */
PP_API int pp_make_hits_from_photons(const pp_hit_record* d_records, int64_t n,
                                     const pp_pmt_target* targets, int32_t n_targets,
                                     const pp_pom_model* pom, int64_t seed, int32_t* d_pmt_id,
                                     float* d_qe_weight, void* stream);

/* pp_make_hits_from_photons for every module kind: POMs as above; a DOM
 * (check_pmt_hit and apply_wl_acceptance, src/dom.jl:96-134) is detected, as
 * PMT 1, when u1 * polymax < poly(cos zenith) and u2 < wl_acc(wavelength),
 * qe weight 1 (the reference defines no QE for DOMs); a multi-PMT module
 * (check_pmt_hit, src/detection.jl:90-131) is hit when u1 <= sum over PMTs of
 * max(direction . axis, 0) * pmt_area / (pi r^2), by the PMT that a cumulative
 * scan of the weights -(rel . axis) picks for u2 (StatsBase 0.34 weighted
 * sample), qe weight = QE(wavelength). */
PP_API int pp_make_hits_from_photons_models(const pp_hit_record* d_records, int64_t n,
                                            const pp_pmt_target* targets, int32_t n_targets,
                                            const pp_detection_models* models, int64_t seed,
                                            int32_t* d_pmt_id, float* d_qe_weight, void* stream);

/* Time residuals of n device hit records: d_tres[i] = time - tgeo[module] - t0
 * (NaN for a module index outside [1, n_targets]), tgeo the host array of
 * per-target geometric times (calc_tgeo / calc_tgeo_tracks for the first
 * source).  The per-hit part of calc_time_residual! (src/calc.jl:270-323). */
PP_API int pp_time_residuals(const pp_hit_record* d_records, int64_t n, const double* tgeo,
                             int32_t n_targets, double t0, double* d_tres, void* stream);

/* ---- diagnostics (no reference counterpart) -------------------------------- */

/* The propagation kernel's one wait, made to run out: one launch on the
 * context's inputs in which every CTA arms its table-staging barrier but
 * issues no copy, so that the wait, bounded to wait_ns (1e3..2e9 ns), expires
 * with nothing in flight; each CTA raises PP_FLAG_TIMEOUT and returns.
 * Returns PP_ERR_TIMEOUT when the bound works (the context stays usable),
 * PP_OK if the wait ended some other way.  Needs a sphere list whose tables
 * are staged in shared memory. */
PP_API int pp_debug_staging_timeout(pp_ctx* ctx, int64_t wait_ns);

/* Philox4x32-10 on the device: out[4*i..4*i+3] = philox(ctr[i], key), n rows.
 * ctr and out are host arrays. */
PP_API int pp_debug_philox(const uint32_t* ctr, int32_t n, uint32_t key0, uint32_t key1,
                           uint32_t* out);

/* Measured FP32 FFMA throughput of `device` (TFLOP/s), the denominator of
 * the propagation kernel's roofline. */
PP_API int pp_measure_fp32_peak(int32_t device, double* tflops);

/* Grid statistics of the last pp_set_targets (cells per axis, items). */
PP_API int pp_grid_info(const pp_ctx* ctx, int32_t dims[3], float cell[3], float origin[3],
                        int64_t* n_items, int64_t* blob_bytes);

#ifdef __cplusplus
}
#endif

#endif /* PP_GB300_H */
