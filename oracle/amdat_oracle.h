/* CPU restatement of AMDAT's hot path: TEST INFRASTRUCTURE ONLY.
 *
 * This oracle is the checker for the GPU engine.  Only tests, the smoke check
 * and the benchmark's CPU-baseline leg may load it; the engine never calls it.
 *
 * Every routine follows the reference function cited beside it (paths relative
 * to the AMDAT source tree).  Two arithmetic modes:
 *   ORC_REF32 - the reference's own arithmetic: FP32 coordinates, FP32
 *               accumulators where the reference has them, the same summation
 *               order, the same libm calls (cosf/sinf/sqrtf/pow).  Its outputs
 *               are pinned against the reference binary's output files.
 *   ORC_F64   - the same enumeration and normalisation with FP64 arithmetic on
 *               the same FP32 inputs: the precision reference for the engine.
 * Coordinates are [frame][atom][3] FP32 arrays.  Lists are ascending atom
 * indices (AMDAT orders list members by trajectory ID, trajectory_list.cpp:315).
 */
#ifndef AMDAT_ORACLE_H
#define AMDAT_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_REF32 = 0, ORC_F64 = 1 };
enum { ORC_LINEAR = 0, ORC_EXPONENTIAL = 1, ORC_SNAPSHOT = 2 };

typedef struct {
  int32_t kind;
  int32_t n_exponentials;
  int32_t n_exponential_steps;
  float exp_base;
  int32_t frt;
  int32_t first_exponent;
  float time_unit;
  int32_t limit; /* System::displacement_limit (control.cpp:1860 'limit') */
} orc_scheme;

/* fills the derived counts of System::System (system.cpp:83-140, :218) */
void orc_scheme_init(orc_scheme* s, int32_t kind, int32_t a, int32_t b, float base,
                     int32_t frt, int32_t first_exponent, float unit);
int32_t orc_n_timesteps(const orc_scheme* s);
int32_t orc_n_timegaps(const orc_scheme* s);
void orc_timelist(const orc_scheme* s, float* out);
void orc_displacement_times(const orc_scheme* s, float* out);
void orc_timegap_weighting(const orc_scheme* s, int32_t fullblock, int32_t* out);
/* System::displacement_list order; arrays may be NULL to count only */
int64_t orc_pairs_list(const orc_scheme* s, int32_t fullblock, int32_t* gap, int32_t* t0, int32_t* t1);
/* System::displacement_loop order (used by coherent ISF) */
int64_t orc_pairs_loop(const orc_scheme* s, int32_t fullblock, int32_t* gap, int32_t* t0, int32_t* t1);

/* Mean_Square_Displacement (mean_square_displacement.cpp:140-180): msd[g] */
void orc_msd(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
             int32_t n_list, int32_t mode, double* msd, double* weighting);
/* Non_Gaussian_Parameter (non_gaussian_parameter.cpp:96-141), incl. its MSD pass */
void orc_ngp(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
             int32_t n_list, int32_t mode, double* ngp);
/* raw moments for the engine's tolerance tests: sum d^2, sum d^4, atom-pair counts */
void orc_disp_moments(const orc_scheme* s, int32_t fullblock, const float* unwrapped,
                      int32_t n_atoms, const int32_t* list, int32_t n_list,
                      double* sum_d2, double* sum_d4, int64_t* count);
/* Incoherent_Scattering_Function (incoherent_scattering_function.cpp:220-299 +
 * correlation_2d.cpp:150-164).  Shell s has vectors kvec_n[3*(off[s]..off[s+1])]
 * (integer lattice), wave vector = n * spacing.  Output corr[g][s]. */
void orc_isfs(const orc_scheme* s, int32_t fullblock, const float* unwrapped, int32_t n_atoms,
              const int32_t* list, int32_t n_list, const int32_t* kvec_n, const int32_t* shell_off,
              int32_t n_shells, float spacing, double box_len, int32_t mode, double* corr);

/* Spatial bins of the wrapped coordinates (Trajectory_List_Bins) and the
 * per-bin displacement analyses (Bin_Static_Analysis / Bin_Dynamics_Analysis) */
void orc_boxify(float* wrapped, int32_t n_frames, int32_t n_atoms, const float* lo, const float* hi);
void orc_assign_bins(const float* wrapped, int32_t n_frames, int32_t n_atoms, int32_t nx, int32_t ny,
                     int32_t nz, const float* lo, const float* hi, int32_t* bins);
void orc_msd_bins(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
                  int32_t n_list, const int32_t* bins, int32_t n_bins, int32_t persistent, int32_t mode,
                  double* msd, double* weighting);
void orc_isfs_bins(const orc_scheme* s, int32_t fullblock, const float* unwrapped, int32_t n_atoms,
                   const int32_t* list, int32_t n_list, const int32_t* kvec_n, const int32_t* off,
                   int32_t n_shells, float spacing, double box_len, const int32_t* bins, int32_t n_bins,
                   int32_t persistent, int32_t mode, double* corr);
void orc_ngp_bins(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
                  int32_t n_list, const int32_t* bins, int32_t n_bins, int32_t persistent, int32_t mode,
                  double* ngp);
void orc_msd2d_bins(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
                    int32_t n_list, int32_t plane, const int32_t* bins, int32_t n_bins, int32_t persistent,
                    int32_t mode, double* msd);
void orc_mean_disp_bins(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
                        int32_t n_list, const int32_t* bins, int32_t n_bins, int32_t persistent, int32_t mode,
                        double* md);
void orc_fast_particles(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
                        int32_t n_list, int32_t gap, float min_u2, int32_t* fast, int32_t* bins);
/* Van_Hove_Self (van_hove_self.cpp:82-103, space_time_correlation_function.cpp:216,345):
 * counts[g][b] raw, weighting[g], and the normalised correlation (REF32). */
void orc_vhs(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
             int32_t n_list, float max_value, int32_t n_bins, int64_t* counts, int64_t* weighting,
             double* corr);
/* Wave_Density (wave_density.cpp:313-365): rho[t][k] (complex, interleaved re/im).
 * REF32: FP32 k.r, cosf/sinf, double accumulation; F64: exact phases 2*pi*n.r/L. */
void orc_rhok(const float* wrapped, int32_t n_atoms, const int32_t* list, int32_t n_list,
              const int32_t* frames, int32_t n_frames, const int32_t* kvec_n, int32_t n_k,
              float spacing, double box_len, int32_t mode, double* rho);
/* Intermediate_Scattering_Function coherent (intermediate_scattering_function.cpp:237-316,
 * 551-566) on full-trajectory rho tables rho1/rho2 [T][k]; corr[g][s]. */
void orc_isf(const orc_scheme* s, int32_t fullblock, const double* rho1, const double* rho2,
             int32_t n_k, const int32_t* shell_off, int32_t n_shells, int32_t n_list,
             int32_t mode, double* corr);
/* Structure_Factor symmetric (structure_factor.cpp:201-285, analysis_onetime.cpp:22-50):
 * complex<float> rho per frame in REF32; S[s]. */
void orc_structure_factor(const orc_scheme* s, int32_t timescheme, const float* wrapped,
                          int32_t n_atoms, const int32_t* list, int32_t n_list,
                          const int32_t* kvec_n, const int32_t* shell_off, int32_t n_shells,
                          float spacing, double box_len, int32_t mode, double* sq);
/* Radial_Distribution_Function symmetric (radial_distribution_function.cpp:32-285):
 * counts[t][b] (ordered pairs i!=j), mean g(r) as written by the reference. */
void orc_structure_factor_bins(const orc_scheme* s, int32_t timescheme, const float* wrapped,
                               int32_t n_atoms, const int32_t* list, int32_t n_list, const int32_t* bins,
                               int32_t n_bins, const int32_t* kvec_n, const int32_t* shell_off,
                               int32_t n_shells, float spacing, double box_len, int32_t mode, double* sq);
void orc_bins_distance(const float* wrapped, int32_t n_frames, int32_t n_atoms, const float* box, int32_t kind,
                       const int32_t* binned, int32_t n_binned, const int32_t* from, int32_t n_from,
                       const float* point, int32_t axis, int32_t direction, float position, float thickness,
                       int32_t n_bins, int32_t* bins);
void orc_rdf(const orc_scheme* s, int32_t timescheme, const float* wrapped, int32_t n_atoms,
             const float* box, const int32_t* list, int32_t n_list, int32_t n_bins,
             float max_distance, int64_t* counts, double* mean_rdf);
/* Distinct van Hove, intended semantics of van_hove_distinct.cpp:183-213 (the reference
 * bins an uninitialised distance): min-image |r_j(t1) - r_i(t0)| over i != j, wrapped
 * coordinates, FP32 arithmetic as RDF. counts[g][b], weighting[g] = sum n(t0)*(n-1). */
void orc_vhd(const orc_scheme* s, int32_t fullblock, const float* wrapped, int32_t n_atoms,
             const float* box, const int32_t* list, int32_t n_list, float max_value,
             int32_t n_bins, int64_t* counts, int64_t* weighting);

/* Timed CPU baseline: MSD + F_s moments over all pairs, FP64, OpenMP over atoms. */
void orc_disp_fs_parallel(const orc_scheme* s, int32_t fullblock, const float* unwrapped,
                          int32_t n_atoms, const int32_t* kvec_n, int32_t n_k, double box_len,
                          int32_t n_threads, double* sum_d2, double* fs_sum);
/* Timed CPU baseline: rho_k for frames, FP64 accumulation, OpenMP over k vectors. */
void orc_rhok_parallel(const float* wrapped, int32_t n_atoms, const int32_t* frames,
                       int32_t n_frames, const int32_t* kvec_n, int32_t n_k, double box_len,
                       int32_t n_threads, double* rho);
void orc_rhok_lattice(const float* wrapped, int32_t n_atoms, const int32_t* frames,
                      int32_t n_frames, const int32_t* kvec_n, int32_t n_k, double box_len,
                      int32_t n_threads, double* rho);

/* Differentiable structure (no reference counterpart; restates the engine's
 * definitions in FP64 from the FP32 wrapped coordinates).
 * orc_gsmooth: h[b] = sum_f sum_{i<j} G(r_b - r_ij), G the normalised Gaussian
 * of width sigma, r_b = (b+1/2) r_max/n_bins, minimum image, pairs with
 * r_ij >= r_max + 6 sigma skipped, bins within ceil(6 sigma/bin) of floor(r_ij/bin).
 * orc_gsmooth_grad: grad[f][i][3] = d(sum_b w[b] h[b]) / dr_i(frames[f]).
 * orc_sk_grad: grad[f][i][3] = d(sum_s w[s] S_raw[s]) / dr_i(frames[f]) with
 * S_raw[s] = sum_f sum_{k in s} |rho_k(f)|^2 / H_s, k = 2 pi n / box_len. */
void orc_gsmooth(const float* wrapped, int32_t n_atoms, const float* box, const int32_t* list,
                 int32_t n_list, const int32_t* frames, int32_t n_frames, double sigma,
                 double r_max, int32_t n_bins, double* h);
void orc_gsmooth_grad(const float* wrapped, int32_t n_atoms, const float* box, const int32_t* list,
                      int32_t n_list, const int32_t* frames, int32_t n_frames, double sigma,
                      double r_max, int32_t n_bins, const double* w, double* grad);
void orc_sk_grad(const float* wrapped, int32_t n_atoms, const int32_t* list, int32_t n_list,
                 const int32_t* frames, int32_t n_frames, const int32_t* kvec_n, int32_t n_k,
                 const int32_t* shell_off, int32_t n_shells, double box_len, const double* w,
                 int32_t n_threads, double* grad);

/* Sibling displacement analyses (same scheduler, other per-atom kernels).
 * orc_msd2d: Mean_Square_Displacement_2D (mean_square_displacement_2d.cpp:114-199):
 *   msd[g] += |dr_plane|^2, |dr_plane| = sqrt(a*a + b*b) in FP32 (coordinate.h:56),
 *   divided by the summed list sizes; plane 0 = xy, 1 = xz, 2 = yz.
 * orc_mean_disp: Mean_Displacement (mean_displacement.cpp:149-199): md[g][3] +=
 *   u(t1) - u(t0) (FP32 Coordinate), divided by the summed list sizes.
 * orc_u2dist: DebyeWaller_Dist (debyewaller_dist.cpp:14-99) and
 *   Displacement_Distribution (displacement_distribution.cpp:17-83) at one gap:
 *   u2 = float(pow(|dr|, 2)), mean and variance of u2 and its histogram of
 *   bins+1 bins of maxvalue/bins (top bin = overflow), all weighted by
 *   1/timegap_weighting(fullblock=1)[gap] and normalised by the reference's
 *   int atomcount (each pair adds n/w, truncated), with FP32 (REF32) or FP64
 *   (F64) sums.
 * mode REF32 = the reference's FP32 accumulators and order; F64 = FP64. */
void orc_msd2d(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
               int32_t n_list, int32_t plane, int32_t mode, double* msd);
void orc_mean_disp(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
                   int32_t n_list, int32_t mode, double* md);
void orc_u2dist(const orc_scheme* s, const float* unwrapped, int32_t n_atoms, const int32_t* list,
                int32_t n_list, int32_t gap, int32_t bins, float maxvalue, int32_t mode,
                double* mean, double* variance, double* dist);

#ifdef __cplusplus
}
#endif
#endif
