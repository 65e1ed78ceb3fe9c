// Time scheme and time-pair scheduler of AMDAT, on the host.
//
// Follows System::System's time line (src/system.cpp:83-140), n_timegaps
// (:218), create_timelist (:3542-3566), displacement_times (:3763-3787),
// timegap_weighting (:4599-4628), displacement_list (:4090-4179) and
// displacement_loop (:3918-3964).  The pair order of both schedulers is kept
// (pairs arrive grouped by gap, in increasing gap), including the 'limit'
// truncation each scheduler applies and the linear scheme's quirk that lag g
// only starts from frames 0..T-2-g.
#include <cmath>
#include <cstring>

#include "engine.h"

namespace amdat {

int32_t scheme_n_timesteps(const amdat_scheme& s) {
  if (s.kind == AMDAT_EXPONENTIAL) return s.n_exponential_steps * s.n_exponentials + 1;
  if (s.kind == AMDAT_LINEAR) return s.n_exponentials + 1;
  return 1;
}

int32_t scheme_n_timegaps(const amdat_scheme& s) {
  return s.n_exponential_steps + s.n_exponentials - 1 + (s.frt ? 0 : 1);
}

void scheme_check(const amdat_scheme& s) {
  AMDAT_REQUIRE(s.kind == AMDAT_LINEAR || s.kind == AMDAT_EXPONENTIAL || s.kind == AMDAT_SNAPSHOT,
                "unknown time scheme kind");
  AMDAT_REQUIRE(s.n_exponentials >= 0 && s.n_exponential_steps >= 0, "negative scheme size");
  AMDAT_REQUIRE(s.limit >= 0, "negative limit");
  AMDAT_REQUIRE((int64_t)s.n_exponentials * (int64_t)s.n_exponential_steps < (1 << 30),
                "time scheme too large");
  if (s.kind == AMDAT_EXPONENTIAL)
    AMDAT_REQUIRE(s.n_exponentials >= 1 && s.n_exponential_steps >= 1,
                  "exponential scheme needs >= 1 block and >= 1 step");
}

static void timelist(const amdat_scheme& s, float* t) {
  int ii = 0;
  float block_start = 0.0f;
  t[0] = 0.0f;
  for (int b = 0; b < s.n_exponentials; ++b) {
    for (int e = 1; e <= s.n_exponential_steps; ++e) {
      ++ii;
      double p = std::pow((double)s.exp_base, (double)(e - 1 + s.first_exponent));
      volatile float prod;  // keep the reference's separate FP32 multiply and add
      if (p <= e)
        prod = (float)e * s.time_unit;
      else
        prod = (float)std::floor(p) * s.time_unit;
      t[ii] = block_start + prod;
    }
    if (s.n_exponential_steps > 0) block_start = t[ii];
  }
}

Pairs scheme_pairs(const amdat_scheme& s, bool fullblock, bool loop_order) {
  const int K = s.n_exponential_steps, I = s.n_exponentials, G = scheme_n_timegaps(s);
  const int T = scheme_n_timesteps(s), frt = s.frt ? 1 : 0, lim = s.limit;
  Pairs p;
  p.gap_first.assign(G + 1, 0);
  auto put = [&](int g, int a, int b) {
    p.gap.push_back(g);
    p.t0.push_back(a);
    p.t1.push_back(b);
  };
  for (int g = 0; g < K; ++g) {
    int count = 0;
    for (int b = 0; b < I; ++b) {
      int a = K * b + frt;
      put(g, a, a + g);
      ++count;
      // displacement_list stops at limit (limit 0 = none); displacement_loop
      // compares count == limit, which never holds for limit 0 either.
      if (lim != 0 && count == lim) break;
    }
  }
  for (int g = K; g < G - 1 + frt; ++g) {
    int count = 0, bg = g - K + 1;
    bool stop = false;
    for (int e = 0; e < (fullblock ? 1 : 0) * (K - 1) + 1 && !stop; ++e) {
      for (int b = 0; b < I - bg; ++b) {
        int a = K * b + e + frt;
        put(g, a, a + K * bg);
        ++count;
        if (lim != 0 && count == lim) {
          stop = true;
          break;
        }
      }
    }
  }
  if (!frt) put(G - 1, 0, T - 1);
  (void)loop_order;  // both schedulers visit the same pairs in the same order
  for (size_t i = 0; i < p.gap.size(); ++i) p.gap_first[p.gap[i] + 1]++;
  for (int g = 0; g < G; ++g) p.gap_first[g + 1] += p.gap_first[g];
  return p;
}

}  // namespace amdat

using namespace amdat;

extern "C" {

amdat_status amdat_scheme_init(amdat_scheme* s, int32_t kind, int32_t a, int32_t b, float base,
                               int32_t frt, int32_t first_exponent, float unit) {
  return guarded([&] {
    AMDAT_REQUIRE(s != nullptr, "null scheme");
    std::memset(s, 0, sizeof(*s));
    s->kind = kind;
    if (kind == AMDAT_LINEAR) {
      AMDAT_REQUIRE(a >= 1, "linear scheme needs n_timesteps >= 1");
      s->n_exponentials = a - 1;
      s->n_exponential_steps = 1;
      s->exp_base = 1.0f;
      s->time_unit = unit;
    } else if (kind == AMDAT_EXPONENTIAL) {
      s->n_exponentials = a;
      s->n_exponential_steps = b;
      s->exp_base = base;
      s->frt = frt;
      s->first_exponent = first_exponent;
      s->time_unit = unit;
    } else if (kind == AMDAT_SNAPSHOT) {
      s->n_exponentials = 1;
      s->n_exponential_steps = 0;
      s->exp_base = 1.0f;
      s->time_unit = 1.0f;
    }
    scheme_check(*s);
  });
}

amdat_status amdat_scheme_counts(const amdat_scheme* s, int32_t fullblock, int32_t loop_order,
                                 int32_t* n_timesteps, int32_t* n_timegaps, int64_t* n_pairs) {
  return guarded([&] {
    AMDAT_REQUIRE(s != nullptr, "null scheme");
    scheme_check(*s);
    if (n_timesteps) *n_timesteps = scheme_n_timesteps(*s);
    if (n_timegaps) *n_timegaps = scheme_n_timegaps(*s);
    if (n_pairs) *n_pairs = (int64_t)scheme_pairs(*s, fullblock != 0, loop_order != 0).gap.size();
  });
}

amdat_status amdat_scheme_times(const amdat_scheme* s, float* tl, float* gap_times) {
  return guarded([&] {
    AMDAT_REQUIRE(s != nullptr, "null scheme");
    scheme_check(*s);
    const int T = scheme_n_timesteps(*s), G = scheme_n_timegaps(*s), K = s->n_exponential_steps;
    std::vector<float> t(T);
    timelist(*s, t.data());
    if (tl) std::memcpy(tl, t.data(), sizeof(float) * T);
    if (gap_times) {
      const int frt = s->frt ? 1 : 0;
      for (int g = 0; g < K && g < G; ++g) gap_times[g] = t[g + frt] - t[frt];
      for (int b = 1; b < s->n_exponentials; ++b) gap_times[b + K - 1] = t[K * b + frt] - t[frt];
      if (!frt && G > 0) gap_times[G - 1] = t[T - 1] - t[0];
    }
  });
}

amdat_status amdat_scheme_weighting(const amdat_scheme* s, int32_t fullblock, int32_t* w) {
  return guarded([&] {
    AMDAT_REQUIRE(s != nullptr && w != nullptr, "null argument");
    scheme_check(*s);
    const int K = s->n_exponential_steps, I = s->n_exponentials, G = scheme_n_timegaps(*s);
    const int lim = s->limit, frt = s->frt ? 1 : 0;
    for (int g = 0; g < K; ++g) w[g] = (lim != 0 && I > lim) ? lim : I;
    for (int g = K; g < G - 1 + frt; ++g) {
      int bg = g - K + 1;
      int v = (I - bg) + (fullblock ? 1 : 0) * (I - bg) * (K - 1) + 1;  // '+1' as in the reference
      w[g] = (lim != 0 && v > lim) ? lim : v;
    }
    if (!frt) w[G - 1] = 1;
  });
}

amdat_status amdat_scheme_pairs(const amdat_scheme* s, int32_t fullblock, int32_t loop_order,
                                int32_t* gap, int32_t* t0, int32_t* t1) {
  return guarded([&] {
    AMDAT_REQUIRE(s != nullptr, "null scheme");
    scheme_check(*s);
    Pairs p = scheme_pairs(*s, fullblock != 0, loop_order != 0);
    const size_t n = p.gap.size();
    if (gap) std::memcpy(gap, p.gap.data(), n * sizeof(int32_t));
    if (t0) std::memcpy(t0, p.t0.data(), n * sizeof(int32_t));
    if (t1) std::memcpy(t1, p.t1.data(), n * sizeof(int32_t));
  });
}

}  // extern "C"
