/* amdat_gb300 - GB300 engine for AMDAT's time-resolved trajectory statistics.
 *
 * C ABI of the engine's hot path.  Plain pointers and sizes, no C++ or CUDA
 * types; every call returns an amdat_status (0 = success) and never exits the
 * process; amdat_last_error() gives the message of the calling thread's last
 * failure.  One context drives one GPU from one host thread; calls issue work
 * on the context's stream and return when their host-visible results are
 * ready (results written to device pointers, AMDAT_OUT_DEVICE, are ready when
 * the stream is).  Caller-owned arrays are never retained.
 *
 * Reference interfaces replaced (paths in the AMDAT source tree):
 *   time scheme + time-pair scheduler  System::System time line (src/system.cpp:83-140),
 *       create_timelist (:3542), displacement_times (:3763), timegap_weighting (:4599),
 *       displacement_list (:4090-4179), displacement_loop (:3918-3964), 'limit' (src/control.cpp:1860)
 *   trajectory store                   Trajectory::unwrapped / coordinates (src/trajectory.h:37-38)
 *   lists                              Static_Trajectory_List / Trajectory_List::listloop
 *                                      (src/trajectory_list.cpp:191-222)
 *   displacement family                Mean_Square_Displacement::listkernel (src/mean_square_displacement.cpp:164),
 *                                      Non_Gaussian_Parameter::listkernel (src/non_gaussian_parameter.cpp:125),
 *                                      Incoherent_Scattering_Function::listkernel (src/incoherent_scattering_function.cpp:272),
 *                                      Van_Hove_Self::listkernel (src/van_hove_self.cpp:98)
 *   Fourier densities                  Wave_Density::analyze / listkernel (src/wave_density.cpp:313-365),
 *                                      Structure_Factor::listkernel (src/structure_factor.cpp:293)
 *   coherent correlator                Intermediate_Scattering_Function::displacementkernel
 *                                      (src/intermediate_scattering_function.cpp:551-566)
 *   static structure factor            Structure_Factor::timekernel (src/structure_factor.cpp:201-230)
 *   pair histograms                    Radial_Distribution_Function::listkernel2 + bin
 *                                      (src/radial_distribution_function.cpp:233-253),
 *                                      Van_Hove_Distinct::listkernel2 (src/van_hove_distinct.cpp:200-213)
 */
#ifndef AMDAT_GB300_H
#define AMDAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  AMDAT_OK = 0,
  AMDAT_ERR_ARGUMENT = 1, /* null pointer, size or index out of range */
  AMDAT_ERR_STATE = 2,    /* call out of order (e.g. no trajectory uploaded) */
  AMDAT_ERR_CUDA = 3,     /* CUDA runtime failure (message has the CUDA error) */
  AMDAT_ERR_NO_DEVICE = 4,
  AMDAT_ERR_MEMORY = 5,   /* device allocation failed */
  AMDAT_ERR_TIMEOUT = 6   /* a bounded device-side wait gave up */
} amdat_status;

/* output placement flag for run calls */
#define AMDAT_OUT_HOST 0
#define AMDAT_OUT_DEVICE 1

/* arithmetic of a run: mixed = FP32 compensated with FP64 final reduction;
 * plain_fp64 = straightforward FP64 kernels (throughput denominator) */
#define AMDAT_MIXED 0
#define AMDAT_PLAIN_FP64 1

typedef struct amdat_ctx amdat_ctx;

const char* amdat_version(void);
const char* amdat_last_error(void);

/* ---------------------------------------------------------------------------
 * Time scheme and time-pair scheduler (host only, no GPU needed)
 * ------------------------------------------------------------------------- */
#define AMDAT_LINEAR 0
#define AMDAT_EXPONENTIAL 1
#define AMDAT_SNAPSHOT 2

typedef struct {
  int32_t kind;                /* AMDAT_LINEAR / AMDAT_EXPONENTIAL / AMDAT_SNAPSHOT */
  int32_t n_exponentials;      /* blocks (linear: n_timesteps - 1) */
  int32_t n_exponential_steps; /* frames per block (linear: 1) */
  float exp_base;
  int32_t frt;
  int32_t first_exponent;
  float time_unit;
  int32_t limit;               /* time pairs per gap cap ('limit'); 0 = none */
} amdat_scheme;

/* Fill a scheme from the arguments of the system block's time line:
 * linear:      a = n_timesteps, unit
 * exponential: a = blocks, b = steps per block, base, frt, first_exponent, unit
 * snapshot:    no arguments.  Replaces System::System (src/system.cpp:83-140). */
amdat_status amdat_scheme_init(amdat_scheme* s, int32_t kind, int32_t a, int32_t b, float base,
                               int32_t frt, int32_t first_exponent, float unit);
/* n_timesteps, n_timegaps (src/system.cpp:218) and the number of time pairs that
 * displacement_list (loop_order = 0) or displacement_loop (loop_order = 1) visits. */
amdat_status amdat_scheme_counts(const amdat_scheme* s, int32_t fullblock, int32_t loop_order,
                                 int32_t* n_timesteps, int32_t* n_timegaps, int64_t* n_pairs);
/* frame times (create_timelist, src/system.cpp:3542) and gap times
 * (displacement_times, src/system.cpp:3763); either pointer may be NULL. */
amdat_status amdat_scheme_times(const amdat_scheme* s, float* timelist, float* gap_times);
/* System::timegap_weighting(bool) (src/system.cpp:4599-4628) */
amdat_status amdat_scheme_weighting(const amdat_scheme* s, int32_t fullblock, int32_t* weighting);
/* the (gap, t0, t1) triples in scheduler order (displacement_list or displacement_loop) */
amdat_status amdat_scheme_pairs(const amdat_scheme* s, int32_t fullblock, int32_t loop_order,
                                int32_t* gap, int32_t* t0, int32_t* t1);

/* ---------------------------------------------------------------------------
 * Context, trajectory store and lists
 * ------------------------------------------------------------------------- */
amdat_status amdat_create(int32_t device, amdat_ctx** out);
amdat_status amdat_destroy(amdat_ctx* ctx);
/* Issue work on an existing cudaStream_t (passed as void*); NULL restores the
 * context's own stream. */
amdat_status amdat_set_stream(amdat_ctx* ctx, void* cuda_stream);
amdat_status amdat_synchronize(amdat_ctx* ctx);
/* number of kernels this context has launched (for launch accounting) */
amdat_status amdat_launch_count(amdat_ctx* ctx, int64_t* count);
/* Per-kernel timing: with enable != 0 every hot kernel launch is bracketed by
 * CUDA events on the context's stream; amdat_profile_kernel returns the number
 * of launches and their total device time (ms) since the last reset.  Kernel
 * names: disp_mixed_kernel, disp_plain_kernel, rhok_list_kernel,
 * rhok_lattice_kernel, rhok_tc_kernel, rhok_plain_kernel, isf_pairs_kernel,
 * sk_frames_kernel, pair_hist_kernel, gsmooth_kernel, gsmooth_adjoint_kernel,
 * sk_adjoint_columns_kernel, sk_adjoint_direct_kernel, disp_axes_kernel, disp_bins_kernel.  (No counterpart in the reference, which times commands
 * with time(NULL), e.g. src/control.cpp:2190-2196.) */
amdat_status amdat_profile_reset(amdat_ctx* ctx, int32_t enable);
amdat_status amdat_profile_kernel(amdat_ctx* ctx, const char* kernel, int64_t* launches,
                                  double* total_ms);

/* Upload a trajectory: host arrays [n_frames][n_atoms][3] of unwrapped
 * coordinates and (optionally) wrapped ones.  With wrapped == NULL the wrapped
 * coordinates are derived as the custom reader does (c = u - L*floor((u-lo)/L),
 * FP32, src/system.cpp read_custom).  box / box_lo: [3] constant box.  The
 * engine keeps unwrapped coordinates re-referenced to frame 0 (FP32) and
 * wrapped ones as FP32 structure-of-arrays planes.  Replaces the per-atom
 * Coordinate arrays of Trajectory (src/trajectory.h:37-38). */
amdat_status amdat_traj_upload(amdat_ctx* ctx, int32_t n_frames, int32_t n_atoms,
                               const float* unwrapped, const float* wrapped, const float* box,
                               const float* box_lo);
/* Same from FP64 host coordinates (re-referencing is then done in FP64). */
amdat_status amdat_traj_upload_f64(amdat_ctx* ctx, int32_t n_frames, int32_t n_atoms,
                                   const double* unwrapped, const double* wrapped,
                                   const float* box, const float* box_lo);
/* Upload from device memory (pointers on this context's GPU) */
amdat_status amdat_traj_upload_device(amdat_ctx* ctx, int32_t n_frames, int32_t n_atoms,
                                      const float* d_unwrapped, const float* box,
                                      const float* box_lo);
/* Register a static list (Static_Trajectory_List): ascending atom indices.
 * Handle 0 is always the list of all atoms. */
amdat_status amdat_list_create(amdat_ctx* ctx, const int32_t* atoms, int32_t n_atoms,
                               int32_t* handle);
amdat_status amdat_list_size(amdat_ctx* ctx, int32_t handle, int32_t* n_atoms);

/* ---------------------------------------------------------------------------
 * Displacement family: MSD, NGP moments, F_s(q,t), G_s(r,t) in one pass
 * ------------------------------------------------------------------------- */
typedef struct {
  int32_t list;           /* list handle */
  int32_t fullblock;      /* cross-block pairs use every in-block offset */
  int32_t precision;      /* AMDAT_MIXED or AMDAT_PLAIN_FP64 */
  /* self intermediate scattering function: shells of integer lattice vectors,
   * wave vector k = 2*pi*n/kvec_period.  n_shells = 0 disables it. */
  int32_t n_shells;
  const int32_t* shell_offsets; /* [n_shells + 1] */
  const int32_t* kvec_n;        /* [3 * shell_offsets[n_shells]] */
  float kvec_period;
  /* self van Hove histogram: n_bins bins of |dr| in [0, bin_max); 0 disables */
  int32_t n_bins;
  float bin_max;
} amdat_disp_request;

/* Runs every time pair of the context's scheme (amdat_set_scheme) over the
 * list.  Outputs, per gap g (n_timegaps rows), any of which may be NULL:
 *   sum_d2[g]      sum over pairs and atoms of |dr|^2
 *   sum_d4[g]      sum of |dr|^4
 *   atom_pairs[g]  number of (atom, time pair) terms
 *   fs_sum[g][s]   sum of the shell mean of cos(k.dr)
 *   gs_counts[g][b] histogram counts (bin = int(|dr| / (bin_max/n_bins)))
 * out_flags = AMDAT_OUT_DEVICE: the five pointers are device pointers.
 * The context keeps the prepared plans of its last eight requests (lists,
 * shells, bins, fullblock), so a repeated request only launches; a new scheme
 * or trajectory upload drops them. */
amdat_status amdat_disp_run(amdat_ctx* ctx, const amdat_disp_request* req, int32_t out_flags,
                            double* sum_d2, double* sum_d4, int64_t* atom_pairs, double* fs_sum,
                            int64_t* gs_counts);
/* Many lists in one persistent launch: outputs are [n_lists][...] stacks of
 * the single-list outputs (req->list is ignored). */
amdat_status amdat_disp_run_lists(amdat_ctx* ctx, const amdat_disp_request* req,
                                  const int32_t* lists, int32_t n_lists, int32_t out_flags,
                                  double* sum_d2, double* sum_d4, int64_t* atom_pairs,
                                  double* fs_sum, int64_t* gs_counts);
amdat_status amdat_set_scheme(amdat_ctx* ctx, const amdat_scheme* scheme);

/* Per-axis displacement sums and the |dr|^2 distribution of one list over the
 * time pairs of the scheme: every gap (gap = -1) or one gap's pairs (the
 * single-gap displacement_list, src/system.cpp:4349-4412).  Per gap g:
 *   axis_sums[g][6]  sums of dx, dy, dz, dx^2, dy^2, dz^2
 *   sum_d4[g]        sum of |dr|^4
 *   atom_pairs[g]    number of (atom, time pair) terms (0 for gaps not run)
 *   d2_counts[g][b]  histogram of u2 = float(|dr|^2) in the reference's FP32
 *                    chain, b = int(u2 / bin_size), the top bin (n_bins - 1)
 *                    collecting everything beyond it; n_bins = 0 disables it.
 * Any output may be NULL.  Replaces the per-atom kernels of
 * Mean_Square_Displacement_2D (src/mean_square_displacement_2d.cpp:143),
 * Mean_Displacement (src/mean_displacement.cpp:163), DebyeWaller_Dist
 * (src/debyewaller_dist.cpp:64) and Displacement_Distribution
 * (src/displacement_distribution.cpp:69). */
amdat_status amdat_disp_axes_run(amdat_ctx* ctx, int32_t list, int32_t fullblock, int32_t gap,
                                 int32_t n_bins, float bin_size, int32_t out_flags,
                                 double* axis_sums, double* sum_d4, int64_t* atom_pairs,
                                 int64_t* d2_counts);

/* Spatial bins (Control::create_bin_list, src/control.cpp:3841-4000).
 * amdat_boxify: System::boxify (src/system.cpp:4799-4870) on the wrapped
 * coordinates: one outside [lo, hi] on an axis moves by hi - lo on that axis.
 * amdat_bins_create: Trajectory_List_Bins (src/trajectory_list_bins.cpp:207-394,
 * 949-1096): per frame, an atom strictly inside the region [lo, hi] gets bin
 * (ix * ny + iy) * nz + iz with ix = int((x - lo + 10 FLT_EPSILON) /
 * (hi - lo + 20 FLT_EPSILON) * nx) (the differences in FP32, the rest in
 * FP64); others none.  The caller applies the region rules (a bound of 0, or
 * one beyond the box, is the box's) and boxifies first, as create_bin_list does.
 * amdat_bins_read: the map [frames][atoms] (-1 = no bin) and/or the members per
 * frame and bin [frames][bins]; either may be NULL. */
amdat_status amdat_boxify(amdat_ctx* ctx, const float lo[3], const float hi[3]);
amdat_status amdat_bins_create(amdat_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, const float lo[3],
                               const float hi[3], int32_t* handle);
amdat_status amdat_bins_read(amdat_ctx* ctx, int32_t handle, int32_t out_flags, int32_t* bins,
                             int64_t* counts);
/* Distance bins (create_bin_list distance trajectory|point|plane,
 * src/control.cpp:3915-3990; Trajectory_List_Bins, src/trajectory_list_bins.cpp:
 * 461-948 and assign_bins_distance_*, :1097-1760), from the wrapped coordinates
 * (boxify first, as create_bin_list does).  Every member of list `binned` gets,
 * in every frame, bin int(length / thickness) when it is below n_bins, else
 * none; atoms outside the list get none.  length, with the reference's FP32
 * chains:
 *   kind 0: the smallest Coordinate::vector_unwrapped length (box of the
 *           context) to a member of list `from` in the same frame, starting
 *           from the box's largest edge;
 *   kind 1: |dist| with dist = r - point, dist -= box * (dist / (box * 0.5)).integer();
 *   kind 2: along `axis` (0 x, 1 y, 2 z), dist = r - position; direction 0
 *           (average): |L * int(dist / (L * 0.5)) - dist| (the quotient in FP64),
 *           1 (above): dist < 0 ? L + dist : dist, 2 (below): dist < 0 ? |dist| : L - dist.
 * The map's bins lie along z (kinds 0, 1) or along the plane's axis (kind 2); the
 * caller applies the reference's limit on n_bins.  Use the handle like
 * amdat_bins_create's. */
amdat_status amdat_bins_distance(amdat_ctx* ctx, int32_t kind, int32_t binned, int32_t from,
                                 const float point[3], int32_t axis, int32_t direction, float position,
                                 float thickness, int32_t n_bins, int32_t* handle);
amdat_status amdat_bins_free(amdat_ctx* ctx, int32_t handle);

/* Fast_Particles (src/fast_particles.cpp; Control::find_fast and
 * find_fast_fixedthreshold, src/control.cpp:3430-3500): over the time pairs of
 * one gap (fullblock 0), the list members whose u2 = float(pow(|dr|, 2)) exceeds
 * min_u2 are fast in the exponential block of the pair's start frame.  The
 * result is an Exptime_Trajectory_List (src/exptime_trajectory_list.cpp): a
 * one-bin map where frame t holds the fast set of block int(float(t - frt) / K).
 * Use it as the bins of amdat_disp_bins_run (static) to analyse the list, and
 * amdat_bins_read for the members per frame; free it with amdat_bins_free. */
amdat_status amdat_fast_particles(amdat_ctx* ctx, int32_t list, int32_t gap, float min_u2, int32_t* handle);

/* A time-dependent list (Trajectory_List with membership per internal time,
 * src/trajectory_list.h:25,58; the analyses iterate the members of the start
 * frame t0, src/trajectory_list.cpp:191-222): the members of frame t are
 * atom_idx[frame_offsets[t] .. frame_offsets[t + 1]) (CSR over the trajectory's
 * frames; order and repeats do not matter).  Returns a one-bin map handle: bin 0
 * holds each frame's members, for amdat_disp_bins_run / amdat_disp_bins_axes_run
 * (persistent 0: members at t0; 1: members at t0 and t1), amdat_bins_read and
 * amdat_bins_free. */
amdat_status amdat_timelist_create(amdat_ctx* ctx, const int32_t* frame_offsets, const int32_t* atom_idx,
                                   int32_t* handle);

/* MSD and NGP moments and F_s of every bin in one pass: the target line "bin_list <bins>
 * <list> [persistence]" of Control::run_analysis (src/control.h:268-380).
 * persistent = 0: Bin_Static_Analysis (src/bin_static_analysis.h:69-111), the
 * list members in the bin at the start frame t0, pairs of the given fullblock;
 * persistent = 1: Bin_Dynamics_Analysis (src/bin_dynamics_analysis.h), members
 * in the bin at t0 and at t1, pairs of fullblock 0.  Per bin b and gap g:
 *   sum_d2[b][g]     sum of |dr|^2
 *   sum_d4[b][g]     sum of |dr|^4 (accumulated only when sum_d4 is given)
 *   count[b][g]      number of (member, time pair) terms
 *   fs_sum[b][g][s]  sum of the shell mean of cos(k.dr), k = 2 pi n / period,
 *                    for up to 8 shells (list mode: every vector of the shell)
 * Any output may be NULL. */
amdat_status amdat_disp_bins_run(amdat_ctx* ctx, int32_t list, int32_t bins, int32_t persistent,
                                 int32_t fullblock, int32_t n_shells, const int32_t* shell_offsets,
                                 const int32_t* kvec, float period, int32_t out_flags, double* sum_d2,
                                 double* sum_d4, int64_t* count, double* fs_sum);
/* Per-axis sums of every bin in one pass (Bin_Static_Analysis /
 * Bin_Dynamics_Analysis of Mean_Square_Displacement_2D, src/mean_square_displacement_2d.cpp,
 * and Mean_Displacement, src/mean_displacement.cpp; fullblock 0):
 *   axis_sums[b][g][6]  sums of dx, dy, dz, dx^2, dy^2, dz^2
 *   count[b][g]         number of (member, time pair) terms */
amdat_status amdat_disp_bins_axes_run(amdat_ctx* ctx, int32_t list, int32_t bins, int32_t persistent,
                                      int32_t out_flags, double* axis_sums, int64_t* count);

/* Prepared displacement runs (many lists, one persistent launch).  A plan
 * builds its item tables on the device once; amdat_disp_plan_run is then pure
 * stream work and does not synchronise.  AMDAT_PLAN_GRAPH captures the run in
 * a CUDA graph (replayed by each plan_run); AMDAT_PLAN_AUTOTUNE times candidate
 * atom-chunk sizes and blocks per SM and keeps the fastest (remembered per
 * process and, when AMDAT_TUNE_CACHE names a file, across processes as JSON
 * lines).  Results stay in the plan until amdat_disp_plan_read.  The plan
 * refers to the context's trajectory, lists and scheme: amdat_disp_plan_run
 * returns AMDAT_ERR_STATE after amdat_set_scheme or after the upload of a
 * trajectory of another shape (a re-upload of the same shape keeps the plan
 * valid and the next run reads the new coordinates).  (The reference runs one
 * Analysis copy per list, e.g. Bin_Static_Analysis,
 * src/bin_static_analysis.h:69-111.) */
#define AMDAT_PLAN_AUTOTUNE 1
#define AMDAT_PLAN_GRAPH 2
/* Lists that overlap (nested lists, bins plus their union, ...) share work:
 * atoms are grouped into membership classes (atoms that belong to exactly the
 * same lists), every class is processed once per time pair, and each list's
 * sums are the sums of its classes (in a fixed order, FP64).  Used when it
 * removes at least a fifth of the atom-pair terms and yields at most four
 * classes per list; AMDAT_PLAN_NO_SHARING keeps one unit of work per list. */
#define AMDAT_PLAN_NO_SHARING 4
typedef struct amdat_disp_plan amdat_disp_plan;
amdat_status amdat_disp_plan_create(amdat_ctx* ctx, const amdat_disp_request* req,
                                    const int32_t* lists, int32_t n_lists, int32_t flags,
                                    amdat_disp_plan** plan);
amdat_status amdat_disp_plan_run(amdat_ctx* ctx, amdat_disp_plan* plan);
amdat_status amdat_disp_plan_read(amdat_ctx* ctx, amdat_disp_plan* plan, int32_t out_flags,
                                  double* sum_d2, double* sum_d4, int64_t* atom_pairs,
                                  double* fs_sum, int64_t* gs_counts);
amdat_status amdat_disp_plan_info(amdat_disp_plan* plan, int32_t* chunk, int32_t* blocks_per_sm,
                                  int64_t* n_items, double* tuned_ms);
/* Work sharing of a plan: the number of work units (membership classes, or
 * the lists themselves) and the atoms streamed per time pair (the sum of the
 * units' sizes, against the sum of the lists' sizes). */
amdat_status amdat_disp_plan_sharing(amdat_disp_plan* plan, int32_t* n_units, int64_t* unit_atoms,
                                     int64_t* list_atoms);
amdat_status amdat_disp_plan_destroy(amdat_ctx* ctx, amdat_disp_plan* plan);

/* ---------------------------------------------------------------------------
 * Fourier densities rho(k,t) = sum_j exp(i 2 pi n.r_j(t) / period)
 * ------------------------------------------------------------------------- */
/* Explicit vector list (e.g. the reference's q-vector shells), frames given.
 * The table stays on the device; returns a handle. */
amdat_status amdat_wave_density(amdat_ctx* ctx, int32_t list, const int32_t* kvec_n, int32_t n_k,
                                float period, const int32_t* frames, int32_t n_frames,
                                int32_t precision, int32_t* handle);
/* Every half-space lattice vector with |k| <= kmax (k = 2 pi n / period), sorted
 * into shells of width dk (shell s: s*dk <= |k| < (s+1)*dk).  Returns the handle,
 * the vector count and the number of shells. */
amdat_status amdat_wave_density_lattice(amdat_ctx* ctx, int32_t list, float kmax, float dk,
                                        float period, const int32_t* frames, int32_t n_frames,
                                        int32_t precision, int32_t* handle, int32_t* n_k,
                                        int32_t* n_shells);
/* Vectors and shell offsets of a lattice density (host arrays sized from the
 * counts above; either may be NULL). */
amdat_status amdat_wave_density_vectors(amdat_ctx* ctx, int32_t handle, int32_t* kvec_n,
                                        int32_t* shell_offsets);
/* Copy rho [n_frames][n_k][2] (FP32 re, im) to host or device memory. */
amdat_status amdat_wave_density_read(amdat_ctx* ctx, int32_t handle, int32_t out_flags,
                                     float* rho);
amdat_status amdat_wave_density_free(amdat_ctx* ctx, int32_t handle);

/* Coherent intermediate scattering function: for every time pair (t0,t1) of
 * the scheme in displacement_loop order, corr_sum[g][s] += sum_{k in shell s}
 * Re(rho1(k,t0) conj(rho2(k,t1))) / H_s.  Both densities must cover every
 * frame 0..n_timesteps-1.  pair_count[g] = number of time pairs of gap g. */
amdat_status amdat_isf_run(amdat_ctx* ctx, int32_t density1, int32_t density2, int32_t fullblock,
                           const int32_t* shell_offsets, int32_t n_shells, int32_t out_flags,
                           double* corr_sum, int64_t* pair_count);
/* Static structure factor: s_sum[s] = sum over the density's frames and the
 * shell's vectors of Re(rho1 conj(rho2)) / H_s. */
/* Structure factor of every bin: the bin_list target of structure_factor
 * (src/control.cpp:2730-2737, Bin_Static_Analysis<Structure_Factor>,
 * src/bin_static_analysis.h:69-111).  Bin b of the map analyses, at each of
 * the given frames, the list members whose bin at that frame is b:
 *   s_sum[b][s] = sum over frames and the shell's vectors of |rho_b(k)|^2 / H_s
 *   n_atoms[b]  = number of (member, frame) terms
 * (S(k) of the bin = s_sum / n_atoms).  k = 2 pi n / period; at most 4096 bins. */
amdat_status amdat_structure_factor_bins(amdat_ctx* ctx, int32_t list, int32_t bins,
                                         const int32_t* kvec_n, int32_t n_k, const int32_t* shell_offsets,
                                         int32_t n_shells, float period, const int32_t* frames,
                                         int32_t n_frames, double* s_sum, int64_t* n_atoms);
amdat_status amdat_structure_factor_run(amdat_ctx* ctx, int32_t density1, int32_t density2,
                                        const int32_t* shell_offsets, int32_t n_shells,
                                        int32_t out_flags, double* s_sum);

/* ---------------------------------------------------------------------------
 * Pair histograms (FP32 arithmetic identical to the reference's, so counts
 * are bit-exact): bin = int(minimage(|r_j - r_i|) / (max_distance/n_bins)).
 * ------------------------------------------------------------------------- */
/* RDF: ordered pairs i in list1, j in list2, i != j, per frame:
 * counts[f][b] for the given frames. */
amdat_status amdat_rdf_run(amdat_ctx* ctx, int32_t list1, int32_t list2, const int32_t* frames,
                           int32_t n_frames, float max_distance, int32_t n_bins, int32_t out_flags,
                           int64_t* counts);
/* Distinct van Hove: for every time pair of the scheme (displacement_list
 * order), ordered pairs i in list1 at t0, j in list2 at t1, i != j:
 * counts[g][b]. */
amdat_status amdat_vhd_run(amdat_ctx* ctx, int32_t list1, int32_t list2, int32_t fullblock,
                           float max_distance, int32_t n_bins, int32_t out_flags, int64_t* counts);

/* ---------------------------------------------------------------------------
 * Differentiable structure (no counterpart in the reference, whose nearest
 * parts are the hard-binned RDF, src/radial_distribution_function.cpp:233-285,
 * and Structure_Factor, src/structure_factor.cpp:201-320).
 * ------------------------------------------------------------------------- */
/* Gaussian-smoothed pair histogram of one list over the given frames:
 * h[b] = sum_f sum_{i<j} exp(-(r_b - r_ij)^2 / 2 sigma^2) / (sqrt(2 pi) sigma),
 * r_b = (b + 1/2) r_max / n_bins, r_ij the minimum-image distance of the wrapped
 * coordinates, pairs with r_ij >= r_max + 6 sigma skipped (r_max + 6 sigma must
 * not exceed half the box).  Bins b within ceil(6 sigma n_bins / r_max) of
 * floor(r_ij n_bins / r_max) receive a pair's terms. */
amdat_status amdat_gsmooth_run(amdat_ctx* ctx, int32_t list, const int32_t* frames, int32_t n_frames,
                               float sigma, float r_max, int32_t n_bins, int32_t out_flags,
                               double* h);
/* Adjoint of amdat_gsmooth_run: given dl_dh[n_bins] = dLoss/dh, writes
 * grad[f][i][3] = dLoss/dr_i(frames[f]) for the list's atoms (FP32).  The pair
 * loop is recomputed.  io_flags = AMDAT_OUT_DEVICE: dl_dh and grad are device
 * pointers. */
amdat_status amdat_gsmooth_adjoint(amdat_ctx* ctx, int32_t list, const int32_t* frames,
                                   int32_t n_frames, float sigma, float r_max, int32_t n_bins,
                                   const double* dl_dh, int32_t io_flags, float* grad);
/* Adjoint of the auto structure factor of one density:
 * S_raw[s] = sum_f sum_{k in shell s} |rho_k(f)|^2 / H_s (what
 * amdat_structure_factor_run(ctx, d, d, ...) gives).  Given dl_ds[n_shells],
 * writes grad[f][i][3] = dLoss/dr_i for the density's frames and list atoms.
 * The phases come from the context's current trajectory, which must hold the
 * coordinates the density was computed from. */
amdat_status amdat_structure_factor_adjoint(amdat_ctx* ctx, int32_t density,
                                            const int32_t* shell_offsets, int32_t n_shells,
                                            const double* dl_ds, int32_t io_flags, float* grad);

/* ---------------------------------------------------------------------------
 * Displacement moments without device allocation (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc where they need an MSD
 * (a memory pool or arena that owns the GPU's memory, plugin hosts that forbid
 * allocation after start-up): per gap of the scheme, sums over every time pair
 * and atom of |dr|^2 and |dr|^4, as amdat_disp_run gives for the list of all
 * atoms.  The caller passes device coordinates [n_frames][n_atoms][3]
 * (unwrapped, FP32), two device output arrays of n_timegaps doubles and a
 * stream (NULL = legacy default stream, the device current on the calling
 * thread).  No context is used and nothing is allocated: the temporaries live
 * in a 16 MiB __device__ array that every GPU loading this library holds until
 * exit.  The work must fit in it: one work item per time pair and atom chunk,
 * about 419k items at most, so a scheme of more than about 419k time pairs
 * (a linear scheme of more than about 915 frames) returns AMDAT_ERR_ARGUMENT.
 * Each call copies its tables from host memory it frees on return, so a stream
 * under capture (or the legacy stream while any capture is active) is refused
 * with AMDAT_ERR_STATE; the first call on a device also looks up the array's
 * address and may load the module.  Calls share the array: calls whose GPU
 * work overlaps race.
 * ------------------------------------------------------------------------- */
amdat_status amdat_disp_moments_noalloc(const amdat_scheme* scheme, int32_t fullblock,
                                        const float* d_xyz, int32_t n_frames, int32_t n_atoms,
                                        void* cuda_stream, double* d_sum_d2, double* d_sum_d4);

/* ---------------------------------------------------------------------------
 * Input scripts: run an AMDAT input file's hot-path commands (system with a
 * custom dump, create_list, limit, msd, ngp, isfs, isf, structure_factor, rdf,
 * vhs, vhd) on one GPU and write the reference's output files.  Replaces
 * Control::Control / execute_commands (src/control.cpp:108, :191) for those
 * commands; q-vector files are read from the prefix in AMDAT_QVECTORS
 * (the reference's compiled-in WV3D).  Errors return a status; the message
 * is in amdat_script_error().
 * ------------------------------------------------------------------------- */
amdat_status amdat_run_script(const char* input_path, int32_t device);
const char* amdat_script_error(void);

#ifdef __cplusplus
}
#endif
#endif /* AMDAT_GB300_H */
