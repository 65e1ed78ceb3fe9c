/* CPU restatement of AMDAT's hot path: TEST INFRASTRUCTURE ONLY (see header).
 * Compile with -ffp-contract=off: the reference is built by g++ on x86-64
 * without FMA contraction, and REF32 mode must reproduce its roundings on any
 * host (aarch64 gcc contracts a*b+c by default). */
#include "amdat_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TWO_PI 6.283185307179586476925286766559

/* ------------------------------------------------------------------------- */
/* time scheme: system.cpp:83-140 (parse), :218 (n_timegaps),                 */
/* :3542-3566 (create_timelist), :3763-3787 (displacement_times)              */
/* ------------------------------------------------------------------------- */

void orc_scheme_init(orc_scheme* s, int32_t kind, int32_t a, int32_t b, float base, int32_t frt,
                     int32_t first_exponent, float unit) {
  memset(s, 0, sizeof(*s));
  s->kind = kind;
  if (kind == ORC_LINEAR) { /* 'linear n_timesteps unit' */
    s->n_exponentials = a - 1;
    s->n_exponential_steps = 1;
    s->exp_base = 1.0f;
    s->frt = 0;
    s->first_exponent = 0;
    s->time_unit = unit;
  } else if (kind == ORC_EXPONENTIAL) {
    s->n_exponentials = a;
    s->n_exponential_steps = b;
    s->exp_base = base;
    s->frt = frt;
    s->first_exponent = first_exponent;
    s->time_unit = unit;
  } else { /* snapshot */
    s->n_exponentials = 1;
    s->n_exponential_steps = 0;
    s->exp_base = 1.0f;
    s->time_unit = 1.0f;
  }
}

int32_t orc_n_timesteps(const orc_scheme* s) {
  if (s->kind == ORC_EXPONENTIAL) return s->n_exponential_steps * s->n_exponentials + 1;
  if (s->kind == ORC_LINEAR) return s->n_exponentials + 1;
  return 1;
}

int32_t orc_n_timegaps(const orc_scheme* s) {
  return s->n_exponential_steps + s->n_exponentials - 1 + (s->frt ? 0 : 1);
}

void orc_timelist(const orc_scheme* s, float* t) {
  int ii = 0;
  float block_start = 0.0f;
  t[0] = 0.0f;
  for (int b = 0; b < s->n_exponentials; ++b) {
    for (int e = 1; e <= s->n_exponential_steps; ++e) {
      ++ii;
      double p = pow((double)s->exp_base, (double)(e - 1 + s->first_exponent));
      if (p <= e)
        t[ii] = block_start + (float)e * s->time_unit;
      else
        t[ii] = block_start + (float)floor(p) * s->time_unit;
    }
    block_start = t[ii];
  }
}

void orc_displacement_times(const orc_scheme* s, float* gap) {
  int T = orc_n_timesteps(s), G = orc_n_timegaps(s), K = s->n_exponential_steps;
  float* t = (float*)malloc(sizeof(float) * T);
  orc_timelist(s, t);
  int frt = s->frt ? 1 : 0;
  for (int g = 0; g < K; ++g) gap[g] = t[g + frt] - t[frt];
  for (int b = 1; b < s->n_exponentials; ++b) gap[b + K - 1] = t[K * b + frt] - t[frt];
  if (!frt) gap[G - 1] = t[T - 1] - t[0];
  free(t);
}

/* System::timegap_weighting(bool) (system.cpp:4599-4628), including its '+1'
 * on cross-block gaps (it cancels in the ISF normalisation). */
void orc_timegap_weighting(const orc_scheme* s, int32_t fullblock, int32_t* w) {
  int K = s->n_exponential_steps, I = s->n_exponentials, G = orc_n_timegaps(s);
  int lim = s->limit, frt = s->frt ? 1 : 0;
  for (int g = 0; g < K; ++g) {
    w[g] = I;
    if (w[g] > lim && lim != 0) w[g] = lim;
  }
  for (int g = K; g < G - 1 + frt; ++g) {
    int bg = g - K + 1;
    w[g] = (I - bg) + (fullblock ? 1 : 0) * (I - bg) * (K - 1) + 1;
    if (w[g] > lim && lim != 0) w[g] = lim;
  }
  if (!frt) w[G - 1] = 1;
}

static void put_pair(int64_t n, int32_t* gap, int32_t* t0, int32_t* t1, int g, int a, int b) {
  if (gap) { gap[n] = g; t0[n] = a; t1[n] = b; }
}

/* System::displacement_list(Analysis*, bool) (system.cpp:4090-4179) */
int64_t orc_pairs_list(const orc_scheme* s, int32_t fullblock, int32_t* gap, int32_t* t0,
                       int32_t* t1) {
  int K = s->n_exponential_steps, I = s->n_exponentials, G = orc_n_timegaps(s);
  int T = orc_n_timesteps(s), frt = s->frt ? 1 : 0, lim = s->limit;
  int64_t n = 0;
  for (int g = 0; g < K; ++g) {
    int count = 0, abort_ = 0;
    for (int b = 0; b < I; ++b) {
      if (abort_) continue;
      int a = K * b + frt;
      put_pair(n++, gap, t0, t1, g, a, a + g);
      ++count;
      abort_ = (count == lim && lim != 0);
    }
  }
  for (int g = K; g < G - 1 + frt; ++g) {
    int count = 0, abort_ = 0, bg = g - K + 1;
    for (int e = 0; e < (fullblock ? 1 : 0) * (K - 1) + 1; ++e) {
      if (abort_) continue;
      for (int b = 0; b < I - bg; ++b) {
        if (abort_) continue;
        int a = K * b + e + frt;
        put_pair(n++, gap, t0, t1, g, a, a + K * bg);
        ++count;
        abort_ = (count == lim && lim != 0);
      }
    }
  }
  if (!frt) put_pair(n++, gap, t0, t1, G - 1, 0, T - 1);
  return n;
}

/* System::displacement_loop(Analysis*, Trajectory*, bool) (system.cpp:3918-3964) */
int64_t orc_pairs_loop(const orc_scheme* s, int32_t fullblock, int32_t* gap, int32_t* t0,
                       int32_t* t1) {
  int K = s->n_exponential_steps, I = s->n_exponentials, G = orc_n_timegaps(s);
  int T = orc_n_timesteps(s), frt = s->frt ? 1 : 0, lim = s->limit;
  int64_t n = 0;
  for (int g = 0; g < K; ++g) {
    int count = 0;
    for (int b = 0; b < I; ++b) {
      int a = K * b + frt;
      put_pair(n++, gap, t0, t1, g, a, a + g);
      ++count;
      if (count == lim) break;
    }
  }
  for (int g = K; g < G - 1 + frt; ++g) {
    int count = 0, bg = g - K + 1;
    for (int e = 0; e < (fullblock ? 1 : 0) * (K - 1) + 1; ++e) {
      for (int b = 0; b < I - bg; ++b) {
        int a = K * b + e + frt;
        put_pair(n++, gap, t0, t1, g, a, a + K * bg);
        ++count;
        if (count == lim) break;
      }
      if (count == lim) break;
    }
  }
  if (!frt) put_pair(n++, gap, t0, t1, G - 1, 0, T - 1);
  return n;
}

typedef struct {
  int64_t n;
  int32_t *gap, *t0, *t1;
} pairs_t;

static pairs_t make_pairs(const orc_scheme* s, int fullblock, int loop_order) {
  pairs_t p;
  p.n = loop_order ? orc_pairs_loop(s, fullblock, 0, 0, 0) : orc_pairs_list(s, fullblock, 0, 0, 0);
  size_t bytes = sizeof(int32_t) * (size_t)(p.n > 0 ? p.n : 1);
  p.gap = (int32_t*)malloc(bytes);
  p.t0 = (int32_t*)malloc(bytes);
  p.t1 = (int32_t*)malloc(bytes);
  if (loop_order) orc_pairs_loop(s, fullblock, p.gap, p.t0, p.t1);
  else orc_pairs_list(s, fullblock, p.gap, p.t0, p.t1);
  return p;
}

static void free_pairs(pairs_t* p) { free(p->gap); free(p->t0); free(p->t1); }

/* ------------------------------------------------------------------------- */
/* coordinates                                                               */
/* ------------------------------------------------------------------------- */

#define POS(arr, t, a, c) ((arr)[((size_t)(t) * (size_t)n_atoms + (size_t)(a)) * 3 + (c)])

/* Trajectory::distance (trajectory.cpp:326): |u(t1)-u(t0)| in FP32,
 * Coordinate::length = sqrt(x*x+y*y+z*z) (coordinate.h:55) */
static float dist32(const float* u, int n_atoms, int a, int ta, int tb) {
  float dx = POS(u, tb, a, 0) - POS(u, ta, a, 0);
  float dy = POS(u, tb, a, 1) - POS(u, ta, a, 1);
  float dz = POS(u, tb, a, 2) - POS(u, ta, a, 2);
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

static double dist2_64(const float* u, int n_atoms, int a, int ta, int tb) {
  double dx = (double)POS(u, tb, a, 0) - (double)POS(u, ta, a, 0);
  double dy = (double)POS(u, tb, a, 1) - (double)POS(u, ta, a, 1);
  double dz = (double)POS(u, tb, a, 2) - (double)POS(u, ta, a, 2);
  return dx * dx + dy * dy + dz * dz;
}

/* ------------------------------------------------------------------------- */
/* displacement family                                                       */
/* ------------------------------------------------------------------------- */

/* Membership of a time-dependent list (a bin of Trajectory_List_Bins intersected
 * with a static list): the atoms in bin `bin` at the start frame t0
 * (Bin_Static_Analysis, src/bin_static_analysis.h:69-111), or at both t0 and t1
 * (Bin_Dynamics_Analysis with persistence, src/bin_dynamics_analysis.h:
 * list_displacementkernel; Trajectory_List::time_intersection,
 * src/trajectory_list.cpp:252-278).  NULL: every list member. */
typedef struct {
  const int32_t* bins; /* [frames][atoms] flat bin or -1 */
  int32_t bin;
  int32_t persistent;
} member_t;

static int is_member(const member_t* f, int n_atoms, int a, int ta, int tb) {
  if (!f) return 1;
  if (f->bins[(size_t)ta * n_atoms + a] != f->bin) return 0;
  return !f->persistent || f->bins[(size_t)tb * n_atoms + a] == f->bin;
}

/* Mean_Square_Displacement::list_displacementkernel / listkernel
 * (src/mean_square_displacement.cpp:147-168): weighting += members at t0 */
static void msd_core(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                     int32_t n_list, int32_t mode, const member_t* f, double* msd, double* weighting) {
  int G = orc_n_timegaps(s);
  pairs_t p = make_pairs(s, 0, 0); /* analyze(): displacement_list(this,false) */
  if (mode == ORC_REF32) {
    float* m = (float*)calloc(G, sizeof(float));
    float* w = (float*)calloc(G, sizeof(float));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      int cnt = 0;
      for (int j = 0; j < n_list; ++j) {
        if (!is_member(f, n_atoms, list[j], p.t0[i], p.t1[i])) continue;
        ++cnt;
        float d = dist32(u, n_atoms, list[j], p.t0[i], p.t1[i]);
        m[g] += d * d;
      }
      w[g] += (float)cnt;
    }
    for (int g = 0; g < G; ++g) {
      m[g] /= (float)w[g];
      msd[g] = m[g];
      if (weighting) weighting[g] = w[g];
    }
    free(m); free(w);
  } else {
    double* m = (double*)calloc(G, sizeof(double));
    double* w = (double*)calloc(G, sizeof(double));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      for (int j = 0; j < n_list; ++j) {
        if (!is_member(f, n_atoms, list[j], p.t0[i], p.t1[i])) continue;
        w[g] += 1.0;
        m[g] += dist2_64(u, n_atoms, list[j], p.t0[i], p.t1[i]);
      }
    }
    for (int g = 0; g < G; ++g) {
      msd[g] = m[g] / w[g];
      if (weighting) weighting[g] = w[g];
    }
    free(m); free(w);
  }
  free_pairs(&p);
}

void orc_msd(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
             int32_t n_list, int32_t mode, double* msd, double* weighting) {
  msd_core(s, u, n_atoms, list, n_list, mode, NULL, msd, weighting);
}

/* Non_Gaussian_Parameter (src/non_gaussian_parameter.cpp:96-141) after its MSD
 * pass (src/control.cpp:3345-3372), both over the same (possibly time-dependent)
 * list: weighting += members at t0 */
static void ngp_core(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                     int32_t n_list, int32_t mode, const member_t* f, double* ngp) {
  int G = orc_n_timegaps(s);
  double* msd = (double*)malloc(sizeof(double) * G);
  msd_core(s, u, n_atoms, list, n_list, mode, f, msd, 0); /* Control::ngp runs MSD first */
  pairs_t p = make_pairs(s, 0, 0);
  if (mode == ORC_REF32) {
    float* q = (float*)calloc(G, sizeof(float));
    long* w = (long*)calloc(G, sizeof(long));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      for (int j = 0; j < n_list; ++j) {
        if (!is_member(f, n_atoms, list[j], p.t0[i], p.t1[i])) continue;
        ++w[g];
        float d = dist32(u, n_atoms, list[j], p.t0[i], p.t1[i]);
        q[g] = (float)((double)q[g] + pow((double)d, 4.0)); /* float += double pow */
      }
    }
    for (int g = 0; g < G; ++g) {
      float m = (float)msd[g];
      double fct = (3.0 / (double)(float)w[g]) / (5 * pow((double)m, 2.0));
      q[g] = (float)((double)q[g] * fct);
      q[g] = (float)((double)q[g] - 1.0);
      ngp[g] = q[g];
    }
    free(q); free(w);
  } else {
    double* q = (double*)calloc(G, sizeof(double));
    double* w = (double*)calloc(G, sizeof(double));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      for (int j = 0; j < n_list; ++j) {
        if (!is_member(f, n_atoms, list[j], p.t0[i], p.t1[i])) continue;
        w[g] += 1.0;
        double d2 = dist2_64(u, n_atoms, list[j], p.t0[i], p.t1[i]);
        q[g] += d2 * d2;
      }
    }
    for (int g = 0; g < G; ++g) ngp[g] = q[g] * (3.0 / w[g]) / (5.0 * msd[g] * msd[g]) - 1.0;
    free(q); free(w);
  }
  free(msd);
  free_pairs(&p);
}

void orc_ngp(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
             int32_t n_list, int32_t mode, double* ngp) {
  ngp_core(s, u, n_atoms, list, n_list, mode, NULL, ngp);
}

void orc_disp_moments(const orc_scheme* s, int32_t fullblock, const float* u, int32_t n_atoms,
                      const int32_t* list, int32_t n_list, double* sum_d2, double* sum_d4,
                      int64_t* count) {
  int G = orc_n_timegaps(s);
  pairs_t p = make_pairs(s, fullblock, 0);
  for (int g = 0; g < G; ++g) { sum_d2[g] = 0; sum_d4[g] = 0; count[g] = 0; }
  for (int64_t i = 0; i < p.n; ++i) {
    int g = p.gap[i];
    count[g] += n_list;
    for (int j = 0; j < n_list; ++j) {
      double d2 = dist2_64(u, n_atoms, list ? list[j] : j, p.t0[i], p.t1[i]);
      sum_d2[g] += d2;
      sum_d4[g] += d2 * d2;
    }
  }
  free_pairs(&p);
}

static void isfs_core(const orc_scheme* s, int32_t fullblock, const float* u, int32_t n_atoms,
                      const int32_t* list, int32_t n_list, const int32_t* kvec_n, const int32_t* off,
                      int32_t n_shells, float spacing, double box_len, int32_t mode, const member_t* f,
                      double* corr) {
  int G = orc_n_timegaps(s);
  pairs_t p = make_pairs(s, fullblock, 0);
  int nk = off[n_shells];
  if (mode == ORC_REF32) {
    /* wave vectors as Wave_Vectors::read_vectors stores them: n * spacing in FP32 */
    float* k = (float*)malloc(sizeof(float) * 3 * (nk > 0 ? nk : 1));
    for (int i = 0; i < 3 * nk; ++i) k[i] = (float)kvec_n[i] * spacing;
    float* c = (float*)calloc((size_t)G * n_shells, sizeof(float));
    float* na = (float*)calloc(G, sizeof(float));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i], ta = p.t0[i], tb = p.t1[i];
      for (int j = 0; j < n_list; ++j) {
        int a = list[j];
        if (!is_member(f, n_atoms, a, ta, tb)) continue;
        na[g] += 1.0f;
        float dx = POS(u, tb, a, 0) - POS(u, ta, a, 0);
        float dy = POS(u, tb, a, 1) - POS(u, ta, a, 1);
        float dz = POS(u, tb, a, 2) - POS(u, ta, a, 2);
        for (int m = 0; m < n_shells; ++m) {
          double tmp = 0;
          int cnt = off[m + 1] - off[m];
          for (int v = off[m]; v < off[m + 1]; ++v) {
            float kr = k[3 * v] * dx + k[3 * v + 1] * dy + k[3 * v + 2] * dz;
            tmp += (double)cosf(kr) / (double)cnt;
          }
          c[(size_t)g * n_shells + m] += (float)tmp;
        }
      }
    }
    for (int g = 0; g < G; ++g)
      for (int m = 0; m < n_shells; ++m) {
        c[(size_t)g * n_shells + m] /= (float)na[g];
        corr[(size_t)g * n_shells + m] = c[(size_t)g * n_shells + m];
      }
    free(k); free(c); free(na);
  } else {
    double* c = (double*)calloc((size_t)G * n_shells, sizeof(double));
    double* na = (double*)calloc(G, sizeof(double));
    double tpl = TWO_PI / box_len;
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i], ta = p.t0[i], tb = p.t1[i];
      for (int j = 0; j < n_list; ++j) {
        int a = list[j];
        if (!is_member(f, n_atoms, a, ta, tb)) continue;
        na[g] += 1.0;
        double dx = (double)POS(u, tb, a, 0) - (double)POS(u, ta, a, 0);
        double dy = (double)POS(u, tb, a, 1) - (double)POS(u, ta, a, 1);
        double dz = (double)POS(u, tb, a, 2) - (double)POS(u, ta, a, 2);
        for (int m = 0; m < n_shells; ++m) {
          double tmp = 0;
          int cnt = off[m + 1] - off[m];
          for (int v = off[m]; v < off[m + 1]; ++v)
            tmp += cos(tpl * (kvec_n[3 * v] * dx + kvec_n[3 * v + 1] * dy + kvec_n[3 * v + 2] * dz));
          c[(size_t)g * n_shells + m] += tmp / cnt;
        }
      }
    }
    for (int g = 0; g < G; ++g)
      for (int m = 0; m < n_shells; ++m)
        corr[(size_t)g * n_shells + m] = c[(size_t)g * n_shells + m] / na[g];
    free(c); free(na);
  }
  free_pairs(&p);
}

void orc_isfs(const orc_scheme* s, int32_t fullblock, const float* u, int32_t n_atoms,
              const int32_t* list, int32_t n_list, const int32_t* kvec_n, const int32_t* off,
              int32_t n_shells, float spacing, double box_len, int32_t mode, double* corr) {
  isfs_core(s, fullblock, u, n_atoms, list, n_list, kvec_n, off, n_shells, spacing, box_len, mode, NULL,
            corr);
}

/* System::boxify (src/system.cpp:4799-4870): a wrapped coordinate outside
 * [lo, hi] on some axis moves by one box length (hi - lo, FP32) on that axis. */
void orc_boxify(float* w, int32_t n_frames, int32_t n_atoms, const float* lo, const float* hi) {
  for (int t = 0; t < n_frames; ++t)
    for (int a = 0; a < n_atoms; ++a) {
      float* c = &w[((size_t)t * n_atoms + a) * 3];
      if (c[0] < lo[0] || c[0] > hi[0] || c[1] < lo[1] || c[1] > hi[1] || c[2] < lo[2] || c[2] > hi[2])
        for (int d = 0; d < 3; ++d) {
          int sh = c[d] > hi[d] ? -1 : (c[d] < lo[d] ? 1 : 0);
          c[d] = c[d] + (hi[d] - lo[d]) * (float)sh;
        }
    }
}

/* Trajectory_List_Bins::assign_bins (src/trajectory_list_bins.cpp:949-1009): an
 * atom strictly inside the region is in bin
 * int((x - lo + 10 FLT_EPSILON) / (hi - lo + 20 FLT_EPSILON) * n) per axis, the
 * differences in FP32 and the rest in FP64; flat bin (ix * ny + iy) * nz + iz,
 * -1 outside. */
void orc_assign_bins(const float* w, int32_t n_frames, int32_t n_atoms, int32_t nx, int32_t ny,
                     int32_t nz, const float* lo, const float* hi, int32_t* bins) {
  const int32_t n[3] = {nx, ny, nz};
  for (int t = 0; t < n_frames; ++t)
    for (int a = 0; a < n_atoms; ++a) {
      const float* c = &w[((size_t)t * n_atoms + a) * 3];
      int32_t* out = &bins[(size_t)t * n_atoms + a];
      int in = 1;
      for (int d = 0; d < 3; ++d) in &= (c[d] < hi[d] && c[d] > lo[d]);
      if (!in) { *out = -1; continue; }
      int ix[3];
      for (int d = 0; d < 3; ++d) {
        float num = c[d] - lo[d], den = hi[d] - lo[d];
        ix[d] = (int)(((double)num + (double)FLT_EPSILON * 10.0) / ((double)den + (double)FLT_EPSILON * 20.0) *
                      (double)(float)n[d]);
      }
      *out = (ix[0] * ny + ix[1]) * nz + ix[2];
    }
}

/* Per bin, the MSD of the list members in that bin (membership at t0, or at t0
 * and t1 with persistence): msd[bin][gap], weighting[bin][gap] */
void orc_msd_bins(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                  int32_t n_list, const int32_t* bins, int32_t n_bins, int32_t persistent, int32_t mode,
                  double* msd, double* weighting) {
  int G = orc_n_timegaps(s);
  for (int b = 0; b < n_bins; ++b) {
    member_t f = {bins, b, persistent};
    msd_core(s, u, n_atoms, list, n_list, mode, &f, msd + (size_t)b * G,
             weighting ? weighting + (size_t)b * G : NULL);
  }
}

/* Per bin, the self-intermediate scattering function: corr[bin][gap][shell].
 * With persistence the pairs are those of displacement_list(this) (fullblock 0),
 * as Bin_Dynamics_Analysis::analyze enumerates them. */
void orc_isfs_bins(const orc_scheme* s, int32_t fullblock, const float* u, int32_t n_atoms,
                   const int32_t* list, int32_t n_list, const int32_t* kvec_n, const int32_t* off,
                   int32_t n_shells, float spacing, double box_len, const int32_t* bins, int32_t n_bins,
                   int32_t persistent, int32_t mode, double* corr) {
  int G = orc_n_timegaps(s);
  for (int b = 0; b < n_bins; ++b) {
    member_t f = {bins, b, persistent};
    isfs_core(s, persistent ? 0 : fullblock, u, n_atoms, list, n_list, kvec_n, off, n_shells, spacing,
              box_len, mode, &f, corr + (size_t)b * G * n_shells);
  }
}

void orc_ngp_bins(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list, int32_t n_list,
                  const int32_t* bins, int32_t n_bins, int32_t persistent, int32_t mode, double* ngp) {
  int G = orc_n_timegaps(s);
  for (int b = 0; b < n_bins; ++b) {
    member_t f = {bins, b, persistent};
    ngp_core(s, u, n_atoms, list, n_list, mode, &f, ngp + (size_t)b * G);
  }
}

/* Fast_Particles::analyze / listkernel (src/fast_particles.cpp): the pairs of one
 * gap (displacement_list(this, gap, false)); a member with
 * float(pow(|dr|, 2)) > min_u2 is fast in block int((float(t0) - float(frt)) / float(K)).
 * fast[block][atom] = 1; then the membership map of the Exptime_Trajectory_List:
 * bins[t][atom] = fast[int(float(t - frt) / float(K))][atom] ? 0 : -1. */
void orc_fast_particles(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                        int32_t n_list, int32_t gap, float min_u2, int32_t* fast, int32_t* bins) {
  int T = orc_n_timesteps(s);
  int K = s->n_exponential_steps, nb = s->n_exponentials;
  memset(fast, 0, sizeof(int32_t) * (size_t)nb * n_atoms);
  pairs_t p = make_pairs(s, 0, 0);
  for (int64_t i = 0; i < p.n; ++i) {
    if (p.gap[i] != gap) continue;
    int blk = (int)(((float)p.t0[i] - (float)s->frt) / (float)K);
    for (int j = 0; j < n_list; ++j) {
      float u2 = (float)pow(dist32(u, n_atoms, list[j], p.t0[i], p.t1[i]), 2.0);
      if (u2 > min_u2 && blk >= 0 && blk < nb) fast[(size_t)blk * n_atoms + list[j]] = 1;
    }
  }
  for (int t = 0; t < T; ++t) {
    int blk = (int)((float)(t - s->frt) / (float)K);
    for (int a = 0; a < n_atoms; ++a)
      bins[(size_t)t * n_atoms + a] = (blk >= 0 && blk < nb && fast[(size_t)blk * n_atoms + a]) ? 0 : -1;
  }
  free_pairs(&p);
}

/* Space_Time_Correlation_Function PI (space_time_correlation_function.cpp:20) */
#define STCF_PI 3.141592653589793238462643383280

void orc_vhs(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
             int32_t n_list, float max_value, int32_t n_bins, int64_t* counts, int64_t* weighting,
             double* corr) {
  int G = orc_n_timegaps(s);
  pairs_t p = make_pairs(s, 0, 0); /* analyze(): displacement_list(this) */
  float bin_size = max_value / (float)n_bins;
  float* c = (float*)calloc((size_t)G * n_bins, sizeof(float));
  int* w = (int*)calloc(G, sizeof(int));
  for (size_t i = 0; i < (size_t)G * n_bins; ++i) counts[i] = 0;
  for (int64_t i = 0; i < p.n; ++i) {
    int g = p.gap[i];
    for (int j = 0; j < n_list; ++j) {
      float d = dist32(u, n_atoms, list[j], p.t0[i], p.t1[i]);
      int b = (int)(d / bin_size);
      if (b >= 0 && b < n_bins) {
        c[(size_t)g * n_bins + b] += 1.0f;
        counts[(size_t)g * n_bins + b]++;
      }
      w[g]++;
    }
  }
  for (int b = 0; b < n_bins; ++b) {
    float rshell = b * bin_size;
    float shellvolume = (float)((4.0 / 3.0) * STCF_PI *
                                (pow(rshell + bin_size, 3.0) - pow(rshell, 3.0)));
    for (int g = 0; g < G; ++g) {
      c[(size_t)g * n_bins + b] /= ((float)w[g] * shellvolume);
      corr[(size_t)g * n_bins + b] = c[(size_t)g * n_bins + b];
    }
  }
  for (int g = 0; g < G; ++g) weighting[g] = w[g];
  free(c); free(w);
  free_pairs(&p);
}

/* ------------------------------------------------------------------------- */
/* Fourier densities                                                         */
/* ------------------------------------------------------------------------- */

void orc_rhok(const float* r, int32_t n_atoms, const int32_t* list, int32_t n_list,
              const int32_t* frames, int32_t n_frames, const int32_t* kvec_n, int32_t n_k,
              float spacing, double box_len, int32_t mode, double* rho) {
  float* k = (float*)malloc(sizeof(float) * 3 * (n_k > 0 ? n_k : 1));
  for (int i = 0; i < 3 * n_k; ++i) k[i] = (float)kvec_n[i] * spacing;
  double tpl = TWO_PI / box_len;
  for (int f = 0; f < n_frames; ++f) {
    int t = frames[f];
    double* out = rho + (size_t)f * n_k * 2;
    for (int v = 0; v < 2 * n_k; ++v) out[v] = 0;
    for (int j = 0; j < n_list; ++j) {
      int a = list[j];
      float x = POS(r, t, a, 0), y = POS(r, t, a, 1), z = POS(r, t, a, 2);
      for (int v = 0; v < n_k; ++v) {
        if (mode == ORC_REF32) {
          float kr = k[3 * v] * x + k[3 * v + 1] * y + k[3 * v + 2] * z;
          out[2 * v] += (double)cosf(kr);
          out[2 * v + 1] += (double)sinf(kr);
        } else {
          double ph = tpl * ((double)kvec_n[3 * v] * x + (double)kvec_n[3 * v + 1] * y +
                             (double)kvec_n[3 * v + 2] * z);
          out[2 * v] += cos(ph);
          out[2 * v + 1] += sin(ph);
        }
      }
    }
  }
  free(k);
}

void orc_isf(const orc_scheme* s, int32_t fullblock, const double* rho1, const double* rho2,
             int32_t n_k, const int32_t* off, int32_t n_shells, int32_t n_list, int32_t mode,
             double* corr) {
  int G = orc_n_timegaps(s);
  pairs_t p = make_pairs(s, fullblock, 1); /* displacement_loop order */
  int32_t* w = (int32_t*)malloc(sizeof(int32_t) * G);
  orc_timegap_weighting(s, fullblock, w);
  if (mode == ORC_REF32) {
    float* c = (float*)calloc((size_t)G * n_shells, sizeof(float));
    float* na = (float*)calloc(G, sizeof(float));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      const double* a = rho1 + (size_t)p.t0[i] * n_k * 2;
      const double* b = rho2 + (size_t)p.t1[i] * n_k * 2;
      for (int m = 0; m < n_shells; ++m) {
        int cnt = off[m + 1] - off[m];
        for (int v = off[m]; v < off[m + 1]; ++v) {
          double val = (a[2 * v] * b[2 * v] + a[2 * v + 1] * b[2 * v + 1]) / (double)(float)cnt;
          c[(size_t)g * n_shells + m] = (float)((double)c[(size_t)g * n_shells + m] + val);
        }
      }
      na[g] += (float)n_list / (float)w[g];
    }
    for (int g = 0; g < G; ++g)
      for (int m = 0; m < n_shells; ++m) {
        c[(size_t)g * n_shells + m] /= (float)(na[g] * (float)w[g]);
        corr[(size_t)g * n_shells + m] = c[(size_t)g * n_shells + m];
      }
    free(c); free(na);
  } else {
    double* c = (double*)calloc((size_t)G * n_shells, sizeof(double));
    double* na = (double*)calloc(G, sizeof(double));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      const double* a = rho1 + (size_t)p.t0[i] * n_k * 2;
      const double* b = rho2 + (size_t)p.t1[i] * n_k * 2;
      for (int m = 0; m < n_shells; ++m) {
        int cnt = off[m + 1] - off[m];
        double acc = 0;
        for (int v = off[m]; v < off[m + 1]; ++v) acc += a[2 * v] * b[2 * v] + a[2 * v + 1] * b[2 * v + 1];
        c[(size_t)g * n_shells + m] += acc / cnt;
      }
      na[g] += n_list; /* the reference's n/w * w cancels to the atom-pair count */
    }
    for (int g = 0; g < G; ++g)
      for (int m = 0; m < n_shells; ++m) corr[(size_t)g * n_shells + m] = c[(size_t)g * n_shells + m] / na[g];
    free(c); free(na);
  }
  free(w);
  free_pairs(&p);
}

/* frames visited by Analysis_Onetime::analyze (analysis_onetime.cpp:22-50) */
static int onetime_frames(const orc_scheme* s, int ts, int* out) {
  int n = 0;
  if (ts == -1) {
    for (int t = 0; t < orc_n_timesteps(s); ++t) out[n++] = t;
  } else if (ts < -1) {
    out[n++] = -ts - 2;
  } else {
    for (int t = ts; t < s->n_exponentials; t += s->n_exponential_steps) out[n++] = t;
  }
  return n;
}

void orc_structure_factor(const orc_scheme* s, int32_t ts, const float* r, int32_t n_atoms,
                          const int32_t* list, int32_t n_list, const int32_t* kvec_n,
                          const int32_t* off, int32_t n_shells, float spacing, double box_len,
                          int32_t mode, double* sq) {
  int T = orc_n_timesteps(s);
  int* fr = (int*)malloc(sizeof(int) * (T + 1));
  int nf = onetime_frames(s, ts, fr);
  int nk = off[n_shells];
  if (mode == ORC_REF32) {
    float* k = (float*)malloc(sizeof(float) * 3 * (nk > 0 ? nk : 1));
    for (int i = 0; i < 3 * nk; ++i) k[i] = (float)kvec_n[i] * spacing;
    float* re = (float*)malloc(sizeof(float) * (nk > 0 ? nk : 1));
    float* im = (float*)malloc(sizeof(float) * (nk > 0 ? nk : 1));
    float* S = (float*)calloc(n_shells, sizeof(float));
    int na = 0;
    for (int f = 0; f < nf; ++f) {
      int t = fr[f];
      for (int v = 0; v < nk; ++v) { re[v] = 0; im[v] = 0; }
      for (int j = 0; j < n_list; ++j) {
        int a = list[j];
        float x = POS(r, t, a, 0), y = POS(r, t, a, 1), z = POS(r, t, a, 2);
        for (int v = 0; v < nk; ++v) {
          float kr = k[3 * v] * x + k[3 * v + 1] * y + k[3 * v + 2] * z;
          re[v] += cosf(kr);
          im[v] += sinf(kr);
        }
      }
      for (int m = 0; m < n_shells; ++m) {
        int cnt = off[m + 1] - off[m];
        for (int v = off[m]; v < off[m + 1]; ++v) S[m] += (re[v] * re[v] + im[v] * im[v]) / (float)cnt;
      }
      na += n_list;
    }
    for (int m = 0; m < n_shells; ++m) {
      if ((float)na != 0) S[m] /= (float)na;
      else S[m] = 0;
      sq[m] = S[m];
    }
    free(k); free(re); free(im); free(S);
  } else {
    double* rho = (double*)malloc(sizeof(double) * 2 * (nk > 0 ? nk : 1));
    double* S = (double*)calloc(n_shells, sizeof(double));
    double na = 0;
    for (int f = 0; f < nf; ++f) {
      orc_rhok(r, n_atoms, list, n_list, &fr[f], 1, kvec_n, nk, spacing, box_len, ORC_F64, rho);
      for (int m = 0; m < n_shells; ++m) {
        int cnt = off[m + 1] - off[m];
        double acc = 0;
        for (int v = off[m]; v < off[m + 1]; ++v) acc += rho[2 * v] * rho[2 * v] + rho[2 * v + 1] * rho[2 * v + 1];
        S[m] += cnt ? acc / cnt : 0;
      }
      na += n_list;
    }
    for (int m = 0; m < n_shells; ++m) sq[m] = na != 0 ? S[m] / na : 0;
    free(rho); free(S);
  }
  free(fr);
}

/* Structure factor of every bin: Bin_Static_Analysis<Structure_Factor>
 * (src/bin_static_analysis.h:69-111, src/control.cpp:2730-2737).  Bin b analyses
 * the time-dependent list (list && bin b): at each frame of the time scheme the
 * list members whose bin at that frame is b (ascending atom order), exactly as
 * orc_structure_factor does for a static list; n_atoms counts the members of
 * each frame.  bins[t][a] (-1 = no bin); sq[bin][shell]. */
void orc_structure_factor_bins(const orc_scheme* s, int32_t ts, const float* r, int32_t n_atoms,
                               const int32_t* list, int32_t n_list, const int32_t* bins, int32_t n_bins,
                               const int32_t* kvec_n, const int32_t* off, int32_t n_shells, float spacing,
                               double box_len, int32_t mode, double* sq) {
  int T = orc_n_timesteps(s);
  int* fr = (int*)malloc(sizeof(int) * (T + 1));
  int nf = onetime_frames(s, ts, fr);
  int nk = off[n_shells];
  int32_t* mem = (int32_t*)malloc(sizeof(int32_t) * (n_list > 0 ? n_list : 1));
  float* k = (float*)malloc(sizeof(float) * 3 * (nk > 0 ? nk : 1));
  for (int i = 0; i < 3 * nk; ++i) k[i] = (float)kvec_n[i] * spacing;
  float* re = (float*)malloc(sizeof(float) * (nk > 0 ? nk : 1));
  float* im = (float*)malloc(sizeof(float) * (nk > 0 ? nk : 1));
  double* rho = (double*)malloc(sizeof(double) * 2 * (nk > 0 ? nk : 1));
  for (int b = 0; b < n_bins; ++b) {
    float Sf[128] = {0};
    double Sd[128] = {0};
    int na = 0;
    for (int f = 0; f < nf; ++f) {
      int t = fr[f], nm = 0;
      for (int j = 0; j < n_list; ++j)
        if (bins[(size_t)t * n_atoms + list[j]] == b) mem[nm++] = list[j];
      if (mode == ORC_REF32) {
        for (int v = 0; v < nk; ++v) { re[v] = 0; im[v] = 0; }
        for (int j = 0; j < nm; ++j) {
          int a = mem[j];
          float x = POS(r, t, a, 0), y = POS(r, t, a, 1), z = POS(r, t, a, 2);
          for (int v = 0; v < nk; ++v) {
            float kr = k[3 * v] * x + k[3 * v + 1] * y + k[3 * v + 2] * z;
            re[v] += cosf(kr);
            im[v] += sinf(kr);
          }
        }
        for (int m = 0; m < n_shells && m < 128; ++m) {
          int cnt = off[m + 1] - off[m];
          for (int v = off[m]; v < off[m + 1]; ++v) Sf[m] += (re[v] * re[v] + im[v] * im[v]) / (float)cnt;
        }
      } else {
        orc_rhok(r, n_atoms, mem, nm, &t, 1, kvec_n, nk, spacing, box_len, ORC_F64, rho);
        for (int m = 0; m < n_shells && m < 128; ++m) {
          int cnt = off[m + 1] - off[m];
          double acc = 0;
          for (int v = off[m]; v < off[m + 1]; ++v) acc += rho[2 * v] * rho[2 * v] + rho[2 * v + 1] * rho[2 * v + 1];
          Sd[m] += cnt ? acc / cnt : 0;
        }
      }
      na += nm;
    }
    for (int m = 0; m < n_shells && m < 128; ++m) {
      if (mode == ORC_REF32) {
        if ((float)na != 0) Sf[m] /= (float)na;
        else Sf[m] = 0;
        sq[(size_t)b * n_shells + m] = Sf[m];
      } else {
        sq[(size_t)b * n_shells + m] = na != 0 ? Sd[m] / na : 0;
      }
    }
  }
  free(fr); free(mem); free(k); free(re); free(im); free(rho);
}

/* Distance bins (Trajectory_List_Bins, src/trajectory_list_bins.cpp): the bin of
 * every list member in every frame from its wrapped (boxified) coordinates, -1
 * for atoms outside the list or beyond the last bin.  The FP32 chains are the
 * reference's, operation by operation.
 *   kind 0, assign_bins_distance_clusters (:1097-1170): the smallest
 *     Coordinate::vector_unwrapped length to a member of `from` at the same frame,
 *     starting from the box's largest edge; bin = int(length / thickness).
 *   kind 1, assign_bins_distance_point (:1321-1420): dist = r - point, then
 *     dist -= box * (dist / (box * 0.5)).integer(); bin = int(|dist| / thickness).
 *   kind 2, assign_bins_distance_plane (:1489-1700): along axis, dist = r - position;
 *     average (direction 0): |L * int(dist / (L * 0.5)) - dist| with the quotient in
 *     double; above (1): dist < 0 ? L + dist : dist; below (2): dist < 0 ? |dist| : L - dist.
 * Bins are along z (kinds 0, 1) or along the plane's axis (kind 2), n_bins of
 * them; the flat index is the bin's index on that axis. */
static float vu_len(float dx, float dy, float dz, const float* box) {
  float p[3] = {dx, dy, dz};
  for (int d = 0; d < 3; ++d) {
    if (p[d] > box[d] / 2) p[d] = p[d] - box[d];
    else if (p[d] < -box[d] / 2) p[d] = p[d] + box[d];
  }
  return sqrtf(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
}

void orc_bins_distance(const float* w, int32_t n_frames, int32_t n_atoms, const float* box, int32_t kind,
                       const int32_t* binned, int32_t n_binned, const int32_t* from, int32_t n_from,
                       const float* point, int32_t axis, int32_t direction, float position, float thickness,
                       int32_t n_bins, int32_t* bins) {
  for (size_t i = 0; i < (size_t)n_frames * n_atoms; ++i) bins[i] = -1;
  const float bmax = box[0] > box[1] ? (box[0] > box[2] ? box[0] : box[2]) : (box[1] > box[2] ? box[1] : box[2]);
  for (int t = 0; t < n_frames; ++t)
    for (int i = 0; i < n_binned; ++i) {
      const int a = binned[i];
      const float* c = &w[((size_t)t * n_atoms + a) * 3];
      float length = 0;
      if (kind == 0) {
        length = bmax;
        for (int j = 0; j < n_from; ++j) {
          const float* q = &w[((size_t)t * n_atoms + from[j]) * 3];
          float tl = vu_len(c[0] - q[0], c[1] - q[1], c[2] - q[2], box);
          length = tl < length ? tl : length;
        }
      } else if (kind == 1) {
        float d[3];
        for (int k = 0; k < 3; ++k) {
          d[k] = c[k] - point[k];
          const float half = box[k] * 0.5f;
          const float q = (float)(int)(d[k] / half);
          d[k] -= box[k] * q;
        }
        length = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      } else {
        const float L = box[axis];
        const float dist = c[axis] - position;
        if (direction == 0) length = fabsf(L * (float)(int)((double)dist / ((double)L * 0.5)) - dist);
        else if (direction == 1) length = dist < 0 ? L + dist : dist;
        else length = dist < 0 ? fabsf(dist) : L - dist;
      }
      const int b = (int)(length / thickness);
      if (b >= 0 && b < n_bins) bins[(size_t)t * n_atoms + a] = b;
    }
}

/* ------------------------------------------------------------------------- */
/* pair histograms                                                           */
/* ------------------------------------------------------------------------- */

/* Coordinate::length_unwrapped (coordinate.cpp:126-137) */
static float min_image_len(float dx, float dy, float dz, const float* box) {
  float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  float bx = box[0] - ax, by = box[1] - ay, bz = box[2] - az;
  float mx = ax < bx ? ax : bx, my = ay < by ? ay : by, mz = az < bz ? az : bz;
  return sqrtf(mx * mx + my * my + mz * mz);
}

#define RDF_PI 3.1459265 /* radial_distribution_function.cpp:11, as written */

void orc_rdf(const orc_scheme* s, int32_t ts, const float* r, int32_t n_atoms, const float* box,
             const int32_t* list, int32_t n_list, int32_t n_bins, float max_distance,
             int64_t* counts, double* mean_rdf) {
  int T = orc_n_timesteps(s);
  int* fr = (int*)malloc(sizeof(int) * (T + 1));
  int nf = onetime_frames(s, ts, fr);
  float bin_size = max_distance / (float)n_bins;
  float* trdf = (float*)calloc((size_t)nf * n_bins, sizeof(float));
  float* mean = (float*)calloc(n_bins, sizeof(float));
  for (size_t i = 0; i < (size_t)nf * n_bins; ++i) counts[i] = 0;
  for (int f = 0; f < nf; ++f) {
    int t = fr[f];
    for (int i = 0; i < n_list; ++i) {
      int a = list[i];
      for (int j = 0; j < n_list; ++j) {
        int b = list[j];
        if (a == b) continue;
        float dx = POS(r, t, b, 0) - POS(r, t, a, 0);
        float dy = POS(r, t, b, 1) - POS(r, t, a, 1);
        float dz = POS(r, t, b, 2) - POS(r, t, a, 2);
        float d = min_image_len(dx, dy, dz, box);
        int bi = (int)(d / bin_size);
        if (bi >= 0 && bi < n_bins) {
          trdf[(size_t)f * n_bins + bi] += 1.0f;
          counts[(size_t)f * n_bins + bi]++;
        }
      }
    }
  }
  int ni_total = 0;
  for (int f = 0; f < nf; ++f) {
    float vol = box[0] * box[1] * box[2];
    float rhoj = (float)n_list / vol;
    ni_total += n_list;
    for (int b = 0; b < n_bins; ++b) {
      float rshell = (float)b * bin_size;
      float shellvolume = (float)((4.0 / 3.0) * RDF_PI * (pow(rshell + bin_size, 3.0) - pow(rshell, 3.0)));
      trdf[(size_t)f * n_bins + b] /= ((float)n_list * rhoj * shellvolume);
      mean[b] += trdf[(size_t)f * n_bins + b] * (float)n_list;
    }
  }
  for (int b = 0; b < n_bins; ++b) {
    mean[b] /= (float)ni_total;
    mean_rdf[b] = mean[b];
  }
  free(fr); free(trdf); free(mean);
}

void orc_vhd(const orc_scheme* s, int32_t fullblock, const float* r, int32_t n_atoms,
             const float* box, const int32_t* list, int32_t n_list, float max_value,
             int32_t n_bins, int64_t* counts, int64_t* weighting) {
  int G = orc_n_timegaps(s);
  pairs_t p = make_pairs(s, fullblock, 0);
  float bin_size = max_value / (float)n_bins;
  for (size_t i = 0; i < (size_t)G * n_bins; ++i) counts[i] = 0;
  for (int g = 0; g < G; ++g) weighting[g] = 0;
  for (int64_t q = 0; q < p.n; ++q) {
    int g = p.gap[q], ta = p.t0[q], tb = p.t1[q];
    weighting[g] += (int64_t)n_list * (n_list - 1);
    for (int i = 0; i < n_list; ++i) {
      int a = list[i];
      for (int j = 0; j < n_list; ++j) {
        int b = list[j];
        if (a == b) continue;
        float dx = POS(r, tb, b, 0) - POS(r, ta, a, 0);
        float dy = POS(r, tb, b, 1) - POS(r, ta, a, 1);
        float dz = POS(r, tb, b, 2) - POS(r, ta, a, 2);
        float d = min_image_len(dx, dy, dz, box);
        int bi = (int)(d / bin_size);
        if (bi >= 0 && bi < n_bins) counts[(size_t)g * n_bins + bi]++;
      }
    }
  }
  free_pairs(&p);
}

/* ------------------------------------------------------------------------- */
/* timed CPU baselines (FP64, OpenMP)                                        */
/* ------------------------------------------------------------------------- */

void orc_disp_fs_parallel(const orc_scheme* s, int32_t fullblock, const float* u,
                          int32_t n_atoms, const int32_t* kvec_n, int32_t n_k, double box_len,
                          int32_t n_threads, double* sum_d2, double* fs_sum) {
  int G = orc_n_timegaps(s);
  double tpl = TWO_PI / box_len;
  pairs_t p = make_pairs(s, fullblock, 0);
  for (int g = 0; g < G; ++g) { sum_d2[g] = 0; fs_sum[g] = 0; }
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  for (int64_t i = 0; i < p.n; ++i) {
    int g = p.gap[i], ta = p.t0[i], tb = p.t1[i];
    double d2acc = 0, fsacc = 0;
#pragma omp parallel for reduction(+ : d2acc, fsacc) schedule(static)
    for (int a = 0; a < n_atoms; ++a) {
      double dx = (double)POS(u, tb, a, 0) - (double)POS(u, ta, a, 0);
      double dy = (double)POS(u, tb, a, 1) - (double)POS(u, ta, a, 1);
      double dz = (double)POS(u, tb, a, 2) - (double)POS(u, ta, a, 2);
      d2acc += dx * dx + dy * dy + dz * dz;
      double f = 0;
      for (int v = 0; v < n_k; ++v)
        f += cos(tpl * (kvec_n[3 * v] * dx + kvec_n[3 * v + 1] * dy + kvec_n[3 * v + 2] * dz));
      fsacc += f;
    }
    sum_d2[g] += d2acc;
    fs_sum[g] += fsacc;
  }
  free_pairs(&p);
}

void orc_rhok_parallel(const float* r, int32_t n_atoms, const int32_t* frames, int32_t n_frames,
                       const int32_t* kvec_n, int32_t n_k, double box_len, int32_t n_threads,
                       double* rho) {
  double tpl = TWO_PI / box_len;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  for (int f = 0; f < n_frames; ++f) {
    int t = frames[f];
    double* out = rho + (size_t)f * n_k * 2;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < n_k; ++v) {
      double re = 0, im = 0;
      double kx = tpl * kvec_n[3 * v], ky = tpl * kvec_n[3 * v + 1], kz = tpl * kvec_n[3 * v + 2];
      for (int a = 0; a < n_atoms; ++a) {
        double ph = kx * POS(r, t, a, 0) + ky * POS(r, t, a, 1) + kz * POS(r, t, a, 2);
        re += cos(ph);
        im += sin(ph);
      }
      out[2 * v] = re;
      out[2 * v + 1] = im;
    }
  }
}

/* rho(k) of integer-lattice vectors in FP64, factored per axis: the density
 * of Wave_Density::listkernel (src/wave_density.cpp:339-365), sum over atoms of
 * exp(i k.r) with r the wrapped coordinate, written as
 *   exp(i k.r) = X_a(nx) Y_a(ny) Z_a(nz),  X_a(n) = exp(i 2 pi n x_a / L)
 * where every table entry is a direct FP64 cos/sin of its own phase and the
 * products and sums are FP64 (relative error ~1e-15 per term against the
 * direct orc_rhok_parallel).  Vectors are grouped by (nx, ny) column, so each
 * column's X Y product is formed once per atom; columns run in parallel.
 * kvec_n entries must satisfy |n| <= nmax on every axis. */
void orc_rhok_lattice(const float* r, int32_t n_atoms, const int32_t* frames, int32_t n_frames,
                      const int32_t* kvec_n, int32_t n_k, double box_len, int32_t n_threads,
                      double* rho) {
  int nmax = 0;
  for (int i = 0; i < 3 * n_k; ++i) nmax = abs(kvec_n[i]) > nmax ? abs(kvec_n[i]) : nmax;
  const int W = 2 * nmax + 1;
  const size_t tab = (size_t)W * n_atoms; /* [axis][n + nmax][atom] re and im planes */
  double* re = (double*)malloc(sizeof(double) * 3 * (tab ? tab : 1));
  double* im = (double*)malloc(sizeof(double) * 3 * (tab ? tab : 1));
  /* vectors sorted by column (nx, ny): counting sort on the column index */
  int32_t* col_start = (int32_t*)calloc((size_t)W * W + 1, sizeof(int32_t));
  int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (n_k > 0 ? n_k : 1));
  for (int v = 0; v < n_k; ++v)
    col_start[(kvec_n[3 * v] + nmax) * W + (kvec_n[3 * v + 1] + nmax) + 1]++;
  for (int c = 0; c < W * W; ++c) col_start[c + 1] += col_start[c];
  {
    int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * ((size_t)W * W + 1));
    memcpy(fill, col_start, sizeof(int32_t) * ((size_t)W * W + 1));
    for (int v = 0; v < n_k; ++v) order[fill[(kvec_n[3 * v] + nmax) * W + (kvec_n[3 * v + 1] + nmax)]++] = v;
    free(fill);
  }
  const double tpl = TWO_PI / box_len;
  const int nth = n_threads > 0 ? n_threads : 1;
  for (int f = 0; f < n_frames; ++f) {
    const int t = frames[f];
#pragma omp parallel for num_threads(nth) schedule(static)
    for (int64_t e = 0; e < (int64_t)3 * W * n_atoms; ++e) {
      const int axis = (int)(e / ((int64_t)W * n_atoms));
      const int n = (int)((e / n_atoms) % W) - nmax;
      const int a = (int)(e % n_atoms);
      const double ph = tpl * (double)n * (double)POS(r, t, a, axis);
      re[e] = cos(ph);
      im[e] = sin(ph);
    }
    double* out = rho + (size_t)f * n_k * 2;
#pragma omp parallel num_threads(nth)
    {
      double* wr = (double*)malloc(sizeof(double) * (n_atoms > 0 ? n_atoms : 1));
      double* wi = (double*)malloc(sizeof(double) * (n_atoms > 0 ? n_atoms : 1));
#pragma omp for schedule(dynamic, 4)
      for (int c = 0; c < W * W; ++c) {
        if (col_start[c + 1] == col_start[c]) continue;
        const double* xr = re + (size_t)(c / W) * n_atoms;
        const double* xi = im + (size_t)(c / W) * n_atoms;
        const double* yr = re + tab + (size_t)(c % W) * n_atoms;
        const double* yi = im + tab + (size_t)(c % W) * n_atoms;
        for (int a = 0; a < n_atoms; ++a) {
          wr[a] = xr[a] * yr[a] - xi[a] * yi[a];
          wi[a] = xr[a] * yi[a] + xi[a] * yr[a];
        }
        for (int i = col_start[c]; i < col_start[c + 1]; ++i) {
          const int v = order[i];
          const double* zr = re + 2 * tab + (size_t)(kvec_n[3 * v + 2] + nmax) * n_atoms;
          const double* zi = im + 2 * tab + (size_t)(kvec_n[3 * v + 2] + nmax) * n_atoms;
          double sr = 0, si = 0;
          for (int a = 0; a < n_atoms; ++a) {
            sr += wr[a] * zr[a] - wi[a] * zi[a];
            si += wr[a] * zi[a] + wi[a] * zr[a];
          }
          out[2 * v] = sr;
          out[2 * v + 1] = si;
        }
      }
      free(wr);
      free(wi);
    }
  }
  free(re);
  free(im);
  free(col_start);
  free(order);
}

/* ------------------------------------------------------------------------- */
/* differentiable structure (FP64; no reference counterpart)                 */
/* ------------------------------------------------------------------------- */
#define SG_CUT 6.0
#define INV_SQRT_2PI 0.39894228040143267794

static double min_image_d(double d, double L) { return d - L * rint(d / L); }

/* span of bins a pair touches, as the engine computes it (FP32 bin width) */
static int sg_span(double sigma, double r_max, int32_t n_bins) {
  float bin = (float)r_max / (float)n_bins;
  return (int)ceil((double)(6.0f * (float)sigma / bin));
}

void orc_gsmooth(const float* r, int32_t n_atoms, const float* box, const int32_t* list,
                 int32_t n_list, const int32_t* frames, int32_t n_frames, double sigma,
                 double r_max, int32_t n_bins, double* h) {
  const double bin = r_max / n_bins, cut = r_max + SG_CUT * sigma;
  const int span = sg_span(sigma, r_max, n_bins);
  for (int b = 0; b < n_bins; ++b) h[b] = 0;
  for (int f = 0; f < n_frames; ++f) {
    int t = frames[f];
    for (int i = 0; i < n_list; ++i)
      for (int j = i + 1; j < n_list; ++j) {
        int a = list[i], c = list[j];
        double d[3], r2 = 0;
        for (int k = 0; k < 3; ++k) {
          d[k] = min_image_d((double)POS(r, t, c, k) - (double)POS(r, t, a, k), box[k]);
          r2 += d[k] * d[k];
        }
        if (r2 >= cut * cut) continue;
        double rr = sqrt(r2);
        int bc = (int)(rr / bin);
        for (int b = bc - span; b <= bc + span; ++b) {
          if (b < 0 || b >= n_bins) continue;
          double x = (b + 0.5) * bin - rr;
          h[b] += INV_SQRT_2PI / sigma * exp(-x * x / (2 * sigma * sigma));
        }
      }
  }
}

void orc_gsmooth_grad(const float* r, int32_t n_atoms, const float* box, const int32_t* list,
                      int32_t n_list, const int32_t* frames, int32_t n_frames, double sigma,
                      double r_max, int32_t n_bins, const double* w, double* grad) {
  const double bin = r_max / n_bins, cut = r_max + SG_CUT * sigma;
  const int span = sg_span(sigma, r_max, n_bins);
  for (int f = 0; f < n_frames; ++f) {
    int t = frames[f];
    for (int i = 0; i < n_list; ++i) {
      double g[3] = {0, 0, 0};
      for (int j = 0; j < n_list; ++j) {
        if (j == i) continue;
        int a = list[i], c = list[j];
        double d[3], r2 = 0;
        for (int k = 0; k < 3; ++k) {
          d[k] = min_image_d((double)POS(r, t, a, k) - (double)POS(r, t, c, k), box[k]);
          r2 += d[k] * d[k];
        }
        if (r2 >= cut * cut || r2 == 0) continue;
        double rr = sqrt(r2), psi = 0;
        int bc = (int)(rr / bin);
        for (int b = bc - span; b <= bc + span; ++b) {
          if (b < 0 || b >= n_bins) continue;
          double x = (b + 0.5) * bin - rr;
          psi += w[b] * x / (sigma * sigma) * INV_SQRT_2PI / sigma * exp(-x * x / (2 * sigma * sigma));
        }
        for (int k = 0; k < 3; ++k) g[k] += psi * d[k] / rr;
      }
      for (int k = 0; k < 3; ++k) grad[((size_t)f * n_list + i) * 3 + k] = g[k];
    }
  }
}

void orc_sk_grad(const float* r, int32_t n_atoms, const int32_t* list, int32_t n_list,
                 const int32_t* frames, int32_t n_frames, const int32_t* kvec_n, int32_t n_k,
                 const int32_t* off, int32_t n_shells, double box_len, const double* w,
                 int32_t n_threads, double* grad) {
  const double tpl = TWO_PI / box_len;
  double* u = (double*)calloc(n_k > 0 ? n_k : 1, sizeof(double));
  for (int s = 0; s < n_shells; ++s) {
    int cnt = off[s + 1] - off[s];
    for (int k = off[s]; k < off[s + 1]; ++k) u[k] = 2.0 * w[s] / cnt;
  }
  double* rho = (double*)malloc(sizeof(double) * 2 * (n_k > 0 ? n_k : 1));
  for (int f = 0; f < n_frames; ++f) {
    int t = frames[f];
#ifdef _OPENMP
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(static)
#endif
    for (int k = 0; k < n_k; ++k) {
      double re = 0, im = 0;
      for (int j = 0; j < n_list; ++j) {
        int a = list[j];
        double ph = tpl * ((double)kvec_n[3 * k] * POS(r, t, a, 0) + (double)kvec_n[3 * k + 1] * POS(r, t, a, 1) +
                           (double)kvec_n[3 * k + 2] * POS(r, t, a, 2));
        re += cos(ph);
        im += sin(ph);
      }
      rho[2 * k] = re;
      rho[2 * k + 1] = im;
    }
#ifdef _OPENMP
#pragma omp parallel for num_threads(n_threads > 0 ? n_threads : 1) schedule(static)
#endif
    for (int j = 0; j < n_list; ++j) {
      int a = list[j];
      double g[3] = {0, 0, 0};
      for (int k = 0; k < n_k; ++k) {
        if (u[k] == 0) continue;
        double ph = tpl * ((double)kvec_n[3 * k] * POS(r, t, a, 0) + (double)kvec_n[3 * k + 1] * POS(r, t, a, 1) +
                           (double)kvec_n[3 * k + 2] * POS(r, t, a, 2));
        double v = u[k] * (rho[2 * k + 1] * cos(ph) - rho[2 * k] * sin(ph)) * tpl;
        for (int c = 0; c < 3; ++c) g[c] += v * kvec_n[3 * k + c];
      }
      for (int c = 0; c < 3; ++c) grad[((size_t)f * n_list + j) * 3 + c] = g[c];
    }
  }
  free(rho);
  free(u);
}

/* ------------------------------------------------------------------------- */
/* sibling displacement analyses                                             */
/* ------------------------------------------------------------------------- */

/* Mean_Square_Displacement_2D (src/mean_square_displacement_2d.cpp:79-199) and
 * Mean_Displacement (src/mean_displacement.cpp:149-199) over a (possibly
 * time-dependent) list: weighting += members at t0 */
static void msd2d_core(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                       int32_t n_list, int32_t plane, int32_t mode, const member_t* f, double* msd) {
  const int G = orc_n_timegaps(s);
  const int ca = plane == 2 ? 1 : 0, cb = plane == 0 ? 1 : 2;
  pairs_t p = make_pairs(s, 0, 0); /* analyze(): displacement_list(this) with fullblock false */
  int64_t* w = (int64_t*)calloc(G, sizeof(int64_t));
  if (f && f->persistent) {
    /* Bin_Dynamics_Analysis never calls analyze(), which would zero the weighting:
     * it starts from initialize()'s system->timegap_weighting() (fullblock default 1,
     * src/mean_square_displacement_2d.cpp:116) and the member counts add to that */
    int32_t* tw = (int32_t*)malloc(sizeof(int32_t) * G);
    orc_timegap_weighting(s, 1, tw);
    for (int g = 0; g < G; ++g) w[g] = tw[g];
    free(tw);
  }
  if (mode == ORC_REF32) {
    float* m = (float*)calloc(G, sizeof(float));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      for (int j = 0; j < n_list; ++j) {
        if (!is_member(f, n_atoms, list[j], p.t0[i], p.t1[i])) continue;
        ++w[g];
        float a = POS(u, p.t1[i], list[j], ca) - POS(u, p.t0[i], list[j], ca);
        float b = POS(u, p.t1[i], list[j], cb) - POS(u, p.t0[i], list[j], cb);
        float d = sqrtf(a * a + b * b);
        m[g] += d * d;
      }
    }
    for (int g = 0; g < G; ++g) msd[g] = m[g] / (float)w[g];
    free(m);
  } else {
    double* m = (double*)calloc(G, sizeof(double));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      for (int j = 0; j < n_list; ++j) {
        if (!is_member(f, n_atoms, list[j], p.t0[i], p.t1[i])) continue;
        ++w[g];
        double a = (double)POS(u, p.t1[i], list[j], ca) - (double)POS(u, p.t0[i], list[j], ca);
        double b = (double)POS(u, p.t1[i], list[j], cb) - (double)POS(u, p.t0[i], list[j], cb);
        m[g] += a * a + b * b;
      }
    }
    for (int g = 0; g < G; ++g) msd[g] = m[g] / (double)w[g];
    free(m);
  }
  free(w);
  free_pairs(&p);
}

void orc_msd2d(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
               int32_t n_list, int32_t plane, int32_t mode, double* msd) {
  msd2d_core(s, u, n_atoms, list, n_list, plane, mode, NULL, msd);
}

static void mean_disp_core(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                           int32_t n_list, int32_t mode, const member_t* f, double* md) {
  const int G = orc_n_timegaps(s);
  pairs_t p = make_pairs(s, 0, 0);
  int64_t* w = (int64_t*)calloc(G, sizeof(int64_t));
  if (mode == ORC_REF32) {
    float* m = (float*)calloc((size_t)G * 3, sizeof(float));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      for (int j = 0; j < n_list; ++j) {
        if (!is_member(f, n_atoms, list[j], p.t0[i], p.t1[i])) continue;
        ++w[g];
        for (int c = 0; c < 3; ++c) m[3 * g + c] += POS(u, p.t1[i], list[j], c) - POS(u, p.t0[i], list[j], c);
      }
    }
    for (int g = 0; g < G; ++g)
      for (int c = 0; c < 3; ++c) md[3 * g + c] = m[3 * g + c] / (float)w[g];
    free(m);
  } else {
    double* m = (double*)calloc((size_t)G * 3, sizeof(double));
    for (int64_t i = 0; i < p.n; ++i) {
      int g = p.gap[i];
      for (int j = 0; j < n_list; ++j) {
        if (!is_member(f, n_atoms, list[j], p.t0[i], p.t1[i])) continue;
        ++w[g];
        for (int c = 0; c < 3; ++c)
          m[3 * g + c] += (double)POS(u, p.t1[i], list[j], c) - (double)POS(u, p.t0[i], list[j], c);
      }
    }
    for (int g = 0; g < G; ++g)
      for (int c = 0; c < 3; ++c) md[3 * g + c] = m[3 * g + c] / (double)w[g];
    free(m);
  }
  free(w);
  free_pairs(&p);
}

void orc_mean_disp(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                   int32_t n_list, int32_t mode, double* md) {
  mean_disp_core(s, u, n_atoms, list, n_list, mode, NULL, md);
}

void orc_msd2d_bins(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list, int32_t n_list,
                    int32_t plane, const int32_t* bins, int32_t n_bins, int32_t persistent, int32_t mode,
                    double* msd) {
  int G = orc_n_timegaps(s);
  for (int b = 0; b < n_bins; ++b) {
    member_t f = {bins, b, persistent};
    msd2d_core(s, u, n_atoms, list, n_list, plane, mode, &f, msd + (size_t)b * G);
  }
}

void orc_mean_disp_bins(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                        int32_t n_list, const int32_t* bins, int32_t n_bins, int32_t persistent, int32_t mode,
                        double* md) {
  int G = orc_n_timegaps(s);
  for (int b = 0; b < n_bins; ++b) {
    member_t f = {bins, b, persistent};
    mean_disp_core(s, u, n_atoms, list, n_list, mode, &f, md + (size_t)b * G * 3);
  }
}

void orc_u2dist(const orc_scheme* s, const float* u, int32_t n_atoms, const int32_t* list,
                int32_t n_list, int32_t gap, int32_t bins, float maxvalue, int32_t mode,
                double* mean_out, double* var_out, double* dist_out) {
  const int G = orc_n_timegaps(s);
  const int nb = bins + 1;
  const float binsize = maxvalue / bins;
  int32_t* tw = (int32_t*)malloc(sizeof(int32_t) * G);
  orc_timegap_weighting(s, 1, tw); /* timegap_weighting() defaults to fullblock = 1 */
  const float w = (float)tw[gap];
  pairs_t p = make_pairs(s, 0, 0); /* displacement_list(this, t, false): gap t's pairs */
  if (mode == ORC_REF32) {
    float mean = 0, sq = 0;
    int count = 0; /* int atomcount: each pair's n / w is added and truncated */
    float* dist = (float*)calloc(nb, sizeof(float));
    for (int64_t i = 0; i < p.n; ++i) {
      if (p.gap[i] != gap) continue;
      count = (int)((float)count + (float)n_list / w);
      for (int j = 0; j < n_list; ++j) {
        float msd = (float)pow(dist32(u, n_atoms, list[j], p.t0[i], p.t1[i]), 2.0);
        mean += msd / w;
        sq += msd * msd / w;
        int idx = (int)(msd / binsize);
        if (idx >= nb) idx = nb - 1;
        dist[idx] += 1.0 / w;
      }
    }
    mean /= count;
    float var = sq / count - mean * mean;
    for (int b = 0; b < nb; ++b) dist_out[b] = dist[b] / count;
    *mean_out = mean;
    *var_out = var;
    free(dist);
  } else {
    /* FP64 sums, the reference's normalisation (int atomcount, 1/w weights) */
    double sum = 0, sum2 = 0;
    int count = 0;
    double* dist = (double*)calloc(nb, sizeof(double));
    for (int64_t i = 0; i < p.n; ++i) {
      if (p.gap[i] != gap) continue;
      count = (int)((float)count + (float)n_list / w);
      for (int j = 0; j < n_list; ++j) {
        float d = dist32(u, n_atoms, list[j], p.t0[i], p.t1[i]);
        float msd = (float)((double)d * (double)d);
        double d2 = dist2_64(u, n_atoms, list[j], p.t0[i], p.t1[i]);
        sum += d2;
        sum2 += d2 * d2;
        int idx = (int)(msd / binsize);
        if (idx >= nb) idx = nb - 1;
        dist[idx] += 1.0;
      }
    }
    double mean = sum / w / count;
    *mean_out = mean;
    *var_out = sum2 / w / count - mean * mean;
    for (int b = 0; b < nb; ++b) dist_out[b] = dist[b] / w / count;
    free(dist);
  }
  free(tw);
  free_pairs(&p);
}
