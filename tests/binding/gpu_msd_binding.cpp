// The reference-side binding of the engine, compiled: a GPU-backed mean-square
// displacement written against AMDAT's own Analysis plugin interface
// (src/analysis.h:62-135) and driven by AMDAT's own Control, System and
// Trajectory_List, with AMDAT's sources unmodified.
//
// Gpu_Mean_Square_Displacement is what a maintainer adds in place of
// Mean_Square_Displacement (src/mean_square_displacement.cpp:140-199): the same
// constructor argument, analyze(Trajectory_List*) as one libamdat_gb300 call
// over the whole time scheme instead of the per-atom listkernel loop, and the
// same write() layout.  System has no accessor for the time scheme's first
// exponent, so the binding infers it from System::show_time (the only time
// line that first exponent produces).
//
// main(): runs an AMDAT input script with AMDAT's Control (the system block and
// list commands), takes the list named on the command line, and writes its MSD
// through the GPU-backed analysis:
//   gpu_msd_binding <script> <list name> <output file>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "amdat_gb300.h"
#include "analysis.h"
#include "control.h"
#include "generated/version.h"
#include "system.h"
#include "trajectory_list.h"

// the two definitions of AMDAT's main translation unit that its library code uses
bool fileoutput = true;
void print_progress(int, int) {}

namespace std {

// Trajectory_List keeps its System in a protected member; a member pointer
// named through a derived class reads it from any list (no reference changes)
struct Trajectory_List_Access : Trajectory_List {
  static System* system_of(Trajectory_List* l) { return l->*(&Trajectory_List_Access::sys); }
};

static void check(amdat_status st) {
  if (st != AMDAT_OK) {
    fprintf(stderr, "amdat_gb300: %s\n", amdat_last_error());
    exit(1);
  }
}

// the first exponent of an exponential scheme: the value whose time line is
// nearest the System's (System::show_time); time lines of neighbouring first
// exponents differ by a factor of the base, so a match within 1e-4 relative
// identifies it whatever the rounding of the two computations
static int show_first_exponent(System* sys) {
  int best = -1;
  double best_err = 1e-4;
  for (int fe = 0; fe < 64; ++fe) {
    amdat_scheme s;
    if (amdat_scheme_init(&s, AMDAT_EXPONENTIAL, sys->show_n_exponentials(), sys->show_n_exponential_steps(),
                          sys->show_exp_base(), sys->show_frt() ? 1 : 0, fe, sys->show_time_unit()) != AMDAT_OK)
      continue;
    std::vector<float> tl(sys->show_n_timesteps()), gaps(sys->show_n_timegaps());
    if (amdat_scheme_times(&s, tl.data(), gaps.data()) != AMDAT_OK) continue;
    double err = 0;
    for (int t = 0; t < sys->show_n_timesteps(); ++t) {
      const double a = tl[t], b = sys->show_time(t);
      err = std::max(err, std::fabs(a - b) / std::max(std::fabs(b), 1e-30));
    }
    if (err < best_err) {
      best_err = err;
      best = fe;
    }
  }
  if (best < 0) {
    fprintf(stderr, "no first exponent reproduces the system's time line\n");
    exit(1);
  }
  return best;
}

// one engine context per System: the unwrapped trajectory [frame][atom][3] and
// the time scheme, uploaded at the first analysis
static amdat_ctx* gpu_context(System* sys) {
  static System* owner = nullptr;
  static amdat_ctx* ctx = nullptr;
  if (ctx && owner == sys) return ctx;
  if (!ctx) check(amdat_create(0, &ctx));
  const int T = sys->show_n_timesteps(), N = sys->show_n_atoms();
  std::vector<float> u((size_t)T * N * 3);
  for (int a = 0; a < N; ++a) {
    const Trajectory* tr = sys->show_trajectory(a);
    for (int t = 0; t < T; ++t) {
      const Coordinate c = tr->show_unwrapped(t);
      float* p = &u[((size_t)t * N + a) * 3];
      p[0] = c.show_x();
      p[1] = c.show_y();
      p[2] = c.show_z();
    }
  }
  const Coordinate L = sys->size();
  const float box[3] = {L.show_x(), L.show_y(), L.show_z()};
  check(amdat_traj_upload(ctx, T, N, u.data(), nullptr, box, nullptr));
  amdat_scheme s;
  if (sys->show_timetype() == "linear")
    check(amdat_scheme_init(&s, AMDAT_LINEAR, T, 1, 1.0f, 0, 0, sys->show_time_unit()));
  else
    check(amdat_scheme_init(&s, AMDAT_EXPONENTIAL, sys->show_n_exponentials(), sys->show_n_exponential_steps(),
                            sys->show_exp_base(), sys->show_frt() ? 1 : 0, show_first_exponent(sys),
                            sys->show_time_unit()));
  s.limit = sys->show_displacement_limit();
  check(amdat_set_scheme(ctx, &s));
  owner = sys;
  return ctx;
}

class Gpu_Mean_Square_Displacement : public Analysis {
  int n_times;
  std::vector<float> msd, weighting, timetable;

 public:
  explicit Gpu_Mean_Square_Displacement(System* sys) {
    system = sys;
    n_times = sys->show_n_timegaps();
    msd.assign(n_times, 0.f);
    weighting.assign(n_times, 0.f);
    float* times = sys->displacement_times();
    timetable.assign(times, times + n_times);
    delete[] times;
  }
  Analysis_Type what_are_you() { return mean_square_displacement; }

  // the list's members at its first time (a static list), every time pair of
  // the scheme (System::displacement_list, fullblock 0), one engine call
  void analyze(Trajectory_List* t_list) {
    amdat_ctx* ctx = gpu_context(system);
    std::vector<int32_t> ids;
    for (int i = 0; i < t_list->show_n_trajectories(0); ++i) ids.push_back((*t_list)(0, i)->show_trajectory_ID());
    int32_t h = 0;
    check(amdat_list_create(ctx, ids.data(), (int32_t)ids.size(), &h));
    amdat_disp_request r = {};
    r.list = h;
    std::vector<double> d2(n_times);
    std::vector<int64_t> w(n_times);
    check(amdat_disp_run(ctx, &r, AMDAT_OUT_HOST, d2.data(), nullptr, w.data(), nullptr, nullptr));
    for (int g = 0; g < n_times; ++g) {
      weighting[g] = (float)w[g];
      msd[g] = w[g] ? (float)(d2[g] / (double)w[g]) : 0.f;
    }
  }

  void write(string filename) const {
    ofstream output(filename.c_str());
    output << "Mean square displacement data created by AMDAT v." << amdat::build::SEMVER << "\n";
    for (int g = 0; g < n_times; ++g) output << timetable[g] << "\t" << msd[g] << "\n";
  }
};

}  // namespace std

int main(int argc, char** argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s <script> <list name> <output>\n", argv[0]);
    return 2;
  }
  std::string* consts = new std::string[1];
  std::string* names = new std::string[1];
  std::Control control(argv[1], consts, names, 0, "");
  std::Trajectory_List* list = control.find_trajectorylist(argv[2]);
  std::System* sys = std::Trajectory_List_Access::system_of(list);
  std::Gpu_Mean_Square_Displacement msd(sys);
  msd.analyze(list);
  msd.write(argv[3]);
  return 0;
}
