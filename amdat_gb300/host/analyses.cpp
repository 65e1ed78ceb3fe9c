// Analysis classes of the host mirror: each analyze() issues one engine call
// for the whole time-pair scheduler and list, then normalises and writes the
// reference's output file format (see amdat_host.h for the reference files).
#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>

#include "amdat_host.h"

namespace amdat_host {

namespace {

// glibc on x86-64 prints the default quiet NaN of 0*inf as "-nan"; write that
// on every host so output files match the reference's
struct Num {
  float v;
};
std::ostream& operator<<(std::ostream& o, Num n) {
  if (std::isnan(n.v)) return o << "-nan";
  return o << n.v;
}

std::ofstream open_out(const std::string& file) {
  std::ofstream out(file.c_str());
  if (!out) throw Error(AMDAT_ERR_ARGUMENT, "Cannot write to filename.");
  return out;
}

struct DispOut {
  std::vector<double> d2, d4, fs;
  std::vector<int64_t> pairs, gs;
};

DispOut disp(System* sys, int list, bool fullblock, const std::vector<int32_t>* kvec,
             const std::vector<int32_t>* off, float period, int n_bins, float bin_max) {
  const int G = sys->n_timegaps();
  amdat_disp_request r{};
  r.list = list;
  r.fullblock = fullblock ? 1 : 0;
  r.precision = AMDAT_MIXED;
  if (kvec && off) {
    r.n_shells = (int32_t)off->size() - 1;
    r.shell_offsets = off->data();
    r.kvec_n = kvec->data();
    r.kvec_period = period;
  }
  r.n_bins = n_bins;
  r.bin_max = bin_max;
  DispOut o;
  o.d2.assign(G, 0);
  o.d4.assign(G, 0);
  o.pairs.assign(G, 0);
  o.fs.assign((size_t)G * std::max(r.n_shells, 1), 0);
  o.gs.assign((size_t)G * std::max(n_bins, 1), 0);
  check(amdat_disp_run(sys->ctx(), &r, AMDAT_OUT_HOST, o.d2.data(), o.d4.data(), o.pairs.data(),
                       r.n_shells ? o.fs.data() : nullptr, n_bins ? o.gs.data() : nullptr),
        "displacement run");
  return o;
}

const double PI_STCF = 3.141592653589793238462643383280;  // space_time_correlation_function.cpp:20
const double PI_RDF = 3.1459265;                          // radial_distribution_function.cpp:11

}  // namespace

void Analysis::analyze(Trajectory_List*, Trajectory_List*) {
  throw Error(AMDAT_ERR_ARGUMENT,
              "Trajectory list targets with two lists not implemented for this analysis method.");
}

// --- MSD -------------------------------------------------------------------
Mean_Square_Displacement::Mean_Square_Displacement(System* sys) { system = sys; }

void Mean_Square_Displacement::analyze(Trajectory_List* list) {
  // analyze(): displacement_list(this, false); msd /= weighting
  DispOut o = disp(system, list->handle(), false, nullptr, nullptr, 1.f, 0, 0.f);
  const int G = system->n_timegaps();
  msd_.assign(G, 0.f);
  weighting_.assign(G, 0.0);
  sum_d4 = o.d4;
  for (int g = 0; g < G; ++g) {
    weighting_[g] = (double)o.pairs[g];
    msd_[g] = (float)(o.d2[g] / (double)o.pairs[g]);
  }
}

// --- spatial bins ------------------------------------------------------------
void Analysis::analyze_bins(Trajectory_List*, Trajectory_List_Bins*, bool) {
  throw Error(AMDAT_ERR_ARGUMENT,
              "bin_list targets and time-dependent lists are supported for msd, msd_2d, mean_displacement, "
              "ngp and isfs by this engine");
}

namespace {
struct BinOut {
  std::vector<double> d2, d4, fs;  // [bin][gap], [bin][gap], [bin][gap][shell]
  std::vector<int64_t> cnt;    // [bin][gap]
};
BinOut disp_bins(System* sys, const Trajectory_List* list, const Trajectory_List_Bins* bins, bool persistent,
                 bool fullblock, const std::vector<int32_t>* kvec, const std::vector<int32_t>* off, float period,
                 bool want_d4 = false) {
  const int G = sys->n_timegaps(), B = bins->n_bins();
  const int S = off ? (int)off->size() - 1 : 0;
  BinOut o;
  o.d2.assign((size_t)B * G, 0.0);
  o.d4.assign((size_t)B * G, 0.0);
  o.cnt.assign((size_t)B * G, 0);
  o.fs.assign((size_t)B * G * std::max(S, 1), 0.0);
  // the engine takes up to 8 shells per pass
  for (int s0 = 0; s0 < std::max(S, 1); s0 += 8) {
    const int ns = std::min(8, S - s0);
    std::vector<int32_t> sub_off, sub_kv;
    std::vector<double> fs;
    if (ns > 0) {
      for (int s = s0; s <= s0 + ns; ++s) sub_off.push_back((*off)[s] - (*off)[s0]);
      sub_kv.assign(kvec->begin() + 3 * (*off)[s0], kvec->begin() + 3 * (*off)[s0 + ns]);
      fs.assign((size_t)B * G * ns, 0.0);
    }
    check(amdat_disp_bins_run(sys->ctx(), list->handle(), bins->handle(), persistent ? 1 : 0, fullblock ? 1 : 0,
                              std::max(ns, 0), ns > 0 ? sub_off.data() : nullptr, ns > 0 ? sub_kv.data() : nullptr,
                              period, AMDAT_OUT_HOST, s0 == 0 ? o.d2.data() : nullptr,
                              s0 == 0 && want_d4 ? o.d4.data() : nullptr, s0 == 0 ? o.cnt.data() : nullptr,
                              ns > 0 ? fs.data() : nullptr),
          "binned displacement run");
    for (int bg = 0; bg < B * G; ++bg)
      for (int s = 0; s < ns; ++s) o.fs[(size_t)bg * S + s0 + s] = fs[(size_t)bg * ns + s];
  }
  return o;
}
}  // namespace

Trajectory_List_Bins::Trajectory_List_Bins(System* sys, int nx, int ny, int nz) : sys_(sys), n_{nx, ny, nz} {
  assign(sys->bounds_lo(), sys->bounds_hi());
}

Trajectory_List_Bins::Trajectory_List_Bins(System* sys, int nx, int ny, int nz, float xlo, float xhi, float ylo,
                                           float yhi, float zlo, float zhi)
    : sys_(sys), n_{nx, ny, nz} {
  // src/trajectory_list_bins.cpp:308-357: a bound of 0, or one beyond the box, is the box's
  const float* blo = sys->bounds_lo();
  const float* bhi = sys->bounds_hi();
  const float ulo[3] = {xlo, ylo, zlo}, uhi[3] = {xhi, yhi, zhi};
  float lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = (ulo[d] == 0 || ulo[d] < blo[d]) ? blo[d] : ulo[d];
    hi[d] = (uhi[d] == 0 || uhi[d] > bhi[d]) ? bhi[d] : uhi[d];
  }
  assign(lo, hi);
}

void Trajectory_List_Bins::assign(const float lo[3], const float hi[3]) {
  if (n_[0] < 1 || n_[1] < 1 || n_[2] < 1) throw Error(AMDAT_ERR_ARGUMENT, "bin counts must be positive");
  check(amdat_boxify(sys_->ctx(), sys_->bounds_lo(), sys_->bounds_hi()), "boxify");
  check(amdat_bins_create(sys_->ctx(), n_[0], n_[1], n_[2], lo, hi, &handle_), "bin list");
}

namespace {
// the bins a distance binning can hold: int(length / thickness) + 1
// (src/trajectory_list_bins.cpp:485-504, 604-700, 790-808)
int distance_bin_limit(float length, float thickness) { return (int)(length / thickness) + 1; }
// half the box diagonal, pow(pow(x, 2) + pow(y, 2) + pow(z, 2), .5) in FP64, stored to FP32
float half_diagonal(const float* lo, const float* hi) {
  double s = 0;
  for (int d = 0; d < 3; ++d) {
    const float h = (hi[d] - lo[d]) / 2;
    s += std::pow(h, 2);
  }
  return (float)std::pow(s, .5);
}
}  // namespace

Trajectory_List_Bins::Trajectory_List_Bins(System* sys, float thickness, int n_bins, Trajectory_List* binning,
                                           Trajectory_List* clustered)
    : sys_(sys), n_{1, 1, 1} {
  if (binning->time_dependent() || clustered->time_dependent())
    throw Error(AMDAT_ERR_ARGUMENT, "distance bin lists take static lists here");
  n_[2] = std::min(n_bins, distance_bin_limit(half_diagonal(sys->bounds_lo(), sys->bounds_hi()), thickness));
  check(amdat_boxify(sys_->ctx(), sys_->bounds_lo(), sys_->bounds_hi()), "boxify");
  check(amdat_bins_distance(sys_->ctx(), 0, binning->handle(), clustered->handle(), nullptr, 0, 0, 0.f, thickness,
                            n_[2], &handle_),
        "distance bin list");
}

Trajectory_List_Bins::Trajectory_List_Bins(System* sys, float thickness, int n_bins, Trajectory_List* binning,
                                           Coord point)
    : sys_(sys), n_{1, 1, 1} {
  if (binning->time_dependent()) throw Error(AMDAT_ERR_ARGUMENT, "distance bin lists take static lists here");
  const float* lo = sys->bounds_lo();
  const float* hi = sys->bounds_hi();
  // Coordinate::operator> : beyond the box on any axis
  if (point.x > hi[0] - lo[0] || point.y > hi[1] - lo[1] || point.z > hi[2] - lo[2])
    throw Error(AMDAT_ERR_ARGUMENT, "point chosen does not lie withing the box dimmensions.");
  n_[2] = std::min(n_bins, distance_bin_limit(half_diagonal(lo, hi), thickness));
  const float p[3] = {point.x, point.y, point.z};
  check(amdat_boxify(sys_->ctx(), lo, hi), "boxify");
  check(amdat_bins_distance(sys_->ctx(), 1, binning->handle(), 0, p, 0, 0, 0.f, thickness, n_[2], &handle_),
        "distance bin list");
}

Trajectory_List_Bins::Trajectory_List_Bins(System* sys, float thickness, int n_bins, Trajectory_List* binning,
                                           const std::string& plane, float position, const std::string& direction)
    : sys_(sys), n_{1, 1, 1} {
  if (binning->time_dependent()) throw Error(AMDAT_ERR_ARGUMENT, "distance bin lists take static lists here");
  const int axis = plane == "x" ? 0 : plane == "y" ? 1 : plane == "z" ? 2 : -1;
  const int dir = direction == "average" ? 0 : direction == "above" ? 1 : direction == "below" ? 2 : -1;
  if (axis < 0) throw Error(AMDAT_ERR_ARGUMENT, "plane " + plane + " not recognized, plane must be x, y, or z.");
  if (dir < 0)
    throw Error(AMDAT_ERR_ARGUMENT,
                "could not recognize direction " + direction + ". valid choices are above, below or average.");
  const float* lo = sys->bounds_lo();
  const float* hi = sys->bounds_hi();
  const float L = hi[axis] - lo[axis];
  if (position > L) throw Error(AMDAT_ERR_ARGUMENT, "plane chosen does not lie within the box dimmensions.");
  n_[axis] = std::min(n_bins, distance_bin_limit(dir == 0 ? L / 2 : L, thickness));
  check(amdat_boxify(sys_->ctx(), lo, hi), "boxify");
  check(amdat_bins_distance(sys_->ctx(), 2, binning->handle(), 0, nullptr, axis, dir, position, thickness,
                            n_[axis], &handle_),
        "distance bin list");
}

Trajectory_List_Bins::Trajectory_List_Bins(System* sys, int one_bin_handle)
    : sys_(sys), n_{1, 1, 1}, handle_(one_bin_handle) {}

Trajectory_List_Bins::~Trajectory_List_Bins() {
  if (handle_) amdat_bins_free(sys_->ctx(), handle_);
}

void Mean_Square_Displacement::analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) {
  const BinOut o = disp_bins(system, list, bins, persistent, false, nullptr, nullptr, 1.f);
  const int G = system->n_timegaps(), B = bins->n_bins();
  bin_msd_.assign(B, std::vector<float>(G, 0.f));
  for (int b = 0; b < B; ++b)
    for (int g = 0; g < G; ++g)  // msd /= weighting; an empty bin gives 0/0
      bin_msd_[b][g] = (float)(o.d2[(size_t)b * G + g] / (double)o.cnt[(size_t)b * G + g]);
}

void Mean_Square_Displacement::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  out << "Mean square displacement data created by AMDAT v." << SEMVER << "\n";
  for (int g = 0; g < system->n_timegaps(); ++g)
    out << system->timegaps()[g] << "\t" << Num{msd_[g]} << "\n";
}

// --- sibling displacement analyses ---------------------------------------
namespace {
struct AxesOut {
  std::vector<double> ax, d4;
  std::vector<int64_t> pairs, counts;
};
AxesOut axes(System* sys, int list, int gap, int n_bins, float bin_size) {
  const int G = sys->n_timegaps();
  AxesOut o;
  o.ax.assign((size_t)G * 6, 0);
  o.d4.assign(G, 0);
  o.pairs.assign(G, 0);
  o.counts.assign((size_t)G * std::max(n_bins, 1), 0);
  check(amdat_disp_axes_run(sys->ctx(), list, 0, gap, n_bins, bin_size, AMDAT_OUT_HOST, o.ax.data(),
                            o.d4.data(), o.pairs.data(), n_bins ? o.counts.data() : nullptr),
        "displacement axes run");
  return o;
}
}  // namespace

Mean_Square_Displacement_2D::Mean_Square_Displacement_2D(System* sys, const std::string& plane)
    : plane_(plane) {
  system = sys;
  if (plane == "xy") a_ = 0, b_ = 1;
  else if (plane == "xz") a_ = 0, b_ = 2;
  else if (plane == "yz") a_ = 1, b_ = 2;
  else throw Error(AMDAT_ERR_ARGUMENT, "Error: plane command " + plane + " not understood.");
}

void Mean_Square_Displacement_2D::analyze(Trajectory_List* list) {
  // displacement_list(this) with fullblock false; msd /= weighting (list sizes summed)
  const AxesOut o = axes(system, list->handle(), -1, 0, 1.f);
  const int G = system->n_timegaps();
  msd_.assign(G, 0.f);
  for (int g = 0; g < G; ++g)
    msd_[g] = (float)((o.ax[(size_t)g * 6 + 3 + a_] + o.ax[(size_t)g * 6 + 3 + b_]) / (double)o.pairs[g]);
}

namespace {
struct BinAxes {
  std::vector<double> ax;  // [bin][gap][6]
  std::vector<int64_t> cnt;
};
BinAxes bin_axes(System* sys, const Trajectory_List* list, const Trajectory_List_Bins* bins, bool persistent) {
  BinAxes o;
  const size_t n = (size_t)bins->n_bins() * sys->n_timegaps();
  o.ax.assign(n * 6, 0.0);
  o.cnt.assign(n, 0);
  check(amdat_disp_bins_axes_run(sys->ctx(), list->handle(), bins->handle(), persistent ? 1 : 0, AMDAT_OUT_HOST,
                                 o.ax.data(), o.cnt.data()),
        "binned displacement axes run");
  return o;
}
}  // namespace

void Mean_Square_Displacement_2D::analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) {
  const BinAxes o = bin_axes(system, list, bins, persistent);
  const int G = system->n_timegaps(), B = bins->n_bins();
  // with persistence the reference never calls analyze(), which would zero the
  // weighting: it starts from initialize()'s timegap_weighting() (fullblock 1,
  // src/mean_square_displacement_2d.cpp:116) and the member counts add to that
  std::vector<int32_t> w0(G, 0);
  if (persistent) check(amdat_scheme_weighting(&system->scheme(), 1, w0.data()), "timegap weighting");
  bin_msd_.assign(B, std::vector<float>(G, 0.f));
  for (int b = 0; b < B; ++b)
    for (int g = 0; g < G; ++g) {
      const size_t i = (size_t)b * G + g;
      bin_msd_[b][g] = (float)((o.ax[i * 6 + 3 + a_] + o.ax[i * 6 + 3 + b_]) / (double)(o.cnt[i] + w0[g]));
    }
}

void Mean_Square_Displacement_2D::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  out << "2-D mean square displacement data for " << plane_ << " plane created by AMDAT v." << SEMVER
      << "\n";
  for (int g = 0; g < system->n_timegaps(); ++g)
    out << system->timegaps()[g] << "\t" << Num{msd_[g]} << "\n";
}

Mean_Displacement::Mean_Displacement(System* sys) { system = sys; }

void Mean_Displacement::analyze(Trajectory_List* list) {
  const AxesOut o = axes(system, list->handle(), -1, 0, 1.f);
  const int G = system->n_timegaps();
  md_.assign((size_t)G * 3, 0.f);
  for (int g = 0; g < G; ++g)
    for (int c = 0; c < 3; ++c) md_[(size_t)g * 3 + c] = (float)(o.ax[(size_t)g * 6 + c] / (double)o.pairs[g]);
}

void Mean_Displacement::analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) {
  const BinAxes o = bin_axes(system, list, bins, persistent);
  const int G = system->n_timegaps(), B = bins->n_bins();
  bin_md_.assign(B, std::vector<float>((size_t)G * 3, 0.f));
  for (int b = 0; b < B; ++b)
    for (int g = 0; g < G; ++g) {
      const size_t i = (size_t)b * G + g;
      for (int c = 0; c < 3; ++c) bin_md_[b][(size_t)g * 3 + c] = (float)(o.ax[i * 6 + c] / (double)o.cnt[i]);
    }
}

void Mean_Displacement::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  out << "Mean displacement data created by AMDAT v." << SEMVER << "\n";
  for (int g = 0; g < system->n_timegaps(); ++g)
    out << system->timegaps()[g] << "\t" << Num{md_[(size_t)g * 3]} << "\t" << Num{md_[(size_t)g * 3 + 1]}
        << "\t" << Num{md_[(size_t)g * 3 + 2]} << "\n";
}

DebyeWaller_Dist::DebyeWaller_Dist(System* sys, int bins, float maxvalue, int time_index)
    : n_bins_(bins + 1), time_index_(time_index), binsize_(maxvalue / (float)bins) {
  system = sys;
  if (bins < 1) throw Error(AMDAT_ERR_ARGUMENT, "need at least one bin");
  if (time_index < 0 || time_index >= sys->n_timegaps())
    throw Error(AMDAT_ERR_ARGUMENT, "Requested timegap out of range.");
  time_ = sys->timegaps()[time_index];
}

void DebyeWaller_Dist::analyze(Trajectory_List* list) {
  // displacement_list(this, t, false); every atom-pair term is weighted by
  // 1/timegap_weighting()[t] (fullblock default 1) and the int atomcount
  // accumulates n/w per pair with truncation, as in the reference
  // (debyewaller_dist.cpp:50-99)
  const AxesOut o = axes(system, list->handle(), time_index_, n_bins_, binsize_);
  std::vector<int32_t> tw(system->n_timegaps());
  check(amdat_scheme_weighting(&system->scheme(), 1, tw.data()), "timegap weighting");
  const float w = (float)tw[time_index_];
  const int n = list->show_n_trajectories();
  const int64_t pairs = n > 0 ? o.pairs[time_index_] / n : 0;
  int atomcount = 0;
  for (int64_t p = 0; p < pairs; ++p) atomcount = (int)((float)atomcount + (float)n / w);
  const size_t g6 = (size_t)time_index_ * 6;
  const double sum_u2 = o.ax[g6 + 3] + o.ax[g6 + 4] + o.ax[g6 + 5];
  const float mean = (float)(sum_u2 / (double)w) / (float)atomcount;
  const float square = (float)(o.d4[time_index_] / (double)w);
  mean_ = mean;
  variance_ = square / (float)atomcount - mean * mean;
  dist_.assign(n_bins_, 0.f);
  for (int b = 0; b < n_bins_; ++b)
    dist_[b] = (float)((double)o.counts[(size_t)time_index_ * n_bins_ + b] / (double)w) / (float)atomcount;
}

void DebyeWaller_Dist::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  out << "MSD distribution created by AMDAT v." << SEMVER << "\n";
  out << "MSD time = " << time_ << "\n";
  out << "Mean_stiffness\t" << Num{mean_} << "\n";
  out << "Variance\t" << Num{variance_} << "\n\n";
  for (int b = 0; b < n_bins_; ++b) out << ((float)b + 0.5) * binsize_ << "\t" << Num{dist_[b]} << "\n";
  out << "Last bin includes overflow.";
}

Displacement_Distribution::Displacement_Distribution(System* sys, float power, int bins, float maxvalue,
                                                     int time_index)
    : DebyeWaller_Dist(sys, bins, maxvalue, time_index), power_(power) {}

void Displacement_Distribution::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  out << "Particle displacement distribution to the " << power_ << " power created by AMDAT v." << SEMVER
      << "\n";
  out << "Last bin includes overflow.";
  out << "time = " << time_ << "\n";
  out << "Mean\t" << Num{mean_} << "\n";
  out << "Variance\t" << Num{variance_} << "\n\n";
  for (int b = 0; b < n_bins_; ++b) out << ((float)b + 0.5) * binsize_ << "\t" << Num{dist_[b]} << "\n";
}

// --- NGP -------------------------------------------------------------------
Non_Gaussian_Parameter::Non_Gaussian_Parameter(System* sys) { system = sys; }

void Non_Gaussian_Parameter::analyze(Trajectory_List* list) {
  DispOut o = disp(system, list->handle(), false, nullptr, nullptr, 1.f, 0, 0.f);
  const int G = system->n_timegaps();
  ngp_.assign(G, 0.f);
  for (int g = 0; g < G; ++g) {
    // alpha2 = 3 <d^4> / (5 <d^2>^2) - 1 (non_gaussian_parameter.cpp:138);
    // 0/0 at gap 0 gives NaN as in the reference
    const double w = (double)o.pairs[g];
    const double msd = o.d2[g] / w;
    ngp_[g] = (float)(o.d4[g] * (3.0 / w) / (5.0 * msd * msd) - 1.0);
  }
}

void Non_Gaussian_Parameter::analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) {
  const BinOut o = disp_bins(system, list, bins, persistent, false, nullptr, nullptr, 1.f, true);
  const int G = system->n_timegaps(), B = bins->n_bins();
  bin_ngp_.assign(B, std::vector<float>(G, 0.f));
  for (int b = 0; b < B; ++b)
    for (int g = 0; g < G; ++g) {
      const size_t i = (size_t)b * G + g;
      const double w = (double)o.cnt[i];
      const double msd = o.d2[i] / w;
      bin_ngp_[b][g] = (float)(o.d4[i] * (3.0 / w) / (5.0 * msd * msd) - 1.0);
    }
}

int Non_Gaussian_Parameter::max() const {
  int best = -1;
  float bv = 0;
  for (int g = 1; g < (int)ngp_.size(); ++g)
    if (ngp_[g] > bv) {
      bv = ngp_[g];
      best = g;
    }
  return best;
}

void Non_Gaussian_Parameter::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  out << "Non-Gaussian parameter data created by AMDAT v." << SEMVER << "\n";
  for (int g = 0; g < system->n_timegaps(); ++g)
    out << system->timegaps()[g] << "\t" << Num{ngp_[g]} << "\n";
}

// --- F_s -------------------------------------------------------------------
Incoherent_Scattering_Function::Incoherent_Scattering_Function(System* sys, const Wave_Vectors* wv,
                                                               int inner, int outer, bool fb)
    : wv_(wv), first_(inner), last_(outer), fullblock_(fb) {
  system = sys;
  if (inner < 0 || outer >= wv->n_shells() || outer < inner)
    throw Error(AMDAT_ERR_ARGUMENT, "wavenumber index out of range");
}

void Incoherent_Scattering_Function::analyze(Trajectory_List* list) {
  std::vector<int32_t> kv, off;
  wv_->shells(first_, last_, kv, off);
  DispOut o = disp(system, list->handle(), fullblock_, &kv, &off, wv_->period(), 0, 0.f);
  const int G = system->n_timegaps(), S = last_ - first_ + 1;
  corr_.assign((size_t)G * S, 0.f);
  for (int g = 0; g < G; ++g)
    for (int s = 0; s < S; ++s)
      corr_[(size_t)g * S + s] = (float)(o.fs[(size_t)g * S + s] / (double)o.pairs[g]);
}

void Incoherent_Scattering_Function::analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins,
                                                  bool persistent) {
  std::vector<int32_t> kv, off;
  wv_->shells(first_, last_, kv, off);
  const BinOut o = disp_bins(system, list, bins, persistent, fullblock_, &kv, &off, wv_->period());
  const int G = system->n_timegaps(), S = last_ - first_ + 1, B = bins->n_bins();
  bin_corr_.assign(B, std::vector<float>((size_t)G * S, 0.f));
  for (int b = 0; b < B; ++b)
    for (int g = 0; g < G; ++g)
      for (int s = 0; s < S; ++s)  // Correlation_2D::postprocess_list: corr / n_atoms
        bin_corr_[b][(size_t)g * S + s] =
            (float)(o.fs[((size_t)b * G + g) * S + s] / (double)o.cnt[(size_t)b * G + g]);
}

static void write_corr2d(const std::string& file, const System* sys, const Wave_Vectors* wv, int first,
                         int last, const std::vector<float>& corr) {
  // Correlation_2D::write (correlation_2d.cpp:475-504)
  std::ofstream out = open_out(file);
  out << "Correlation data created by AMDAT v." << SEMVER << "\n";
  out << "\t";
  for (int m = first; m <= last; ++m) out << wv->approx_wavenumber(m) << "\t";
  out << "\n";
  const int S = last - first + 1;
  for (int g = 0; g < sys->n_timegaps(); ++g) {
    out << sys->timegaps()[g] << "\t";
    for (int s = 0; s < S; ++s) out << Num{corr[(size_t)g * S + s]} << "\t";
    out << "\n";
  }
}

void Incoherent_Scattering_Function::write(const std::string& file) const {
  write_corr2d(file, system, wv_, first_, last_, corr_);
}

// --- van Hove self / distinct ------------------------------------------------
Van_Hove_Self::Van_Hove_Self(System* sys, int n_bins, float max_value) : n_bins_(n_bins) {
  system = sys;
  if (n_bins < 1) throw Error(AMDAT_ERR_ARGUMENT, "need >= 1 bin");
  // initialize(): max_value 0 means half the smallest box length (van_hove_self.cpp:53)
  const Coord s = sys->size();
  max_value_ = max_value == 0 ? std::min(s.x, std::min(s.y, s.z)) / 2 : max_value;
  bin_size_ = max_value_ / (float)n_bins_;
}

static void normalise_stcf(const std::vector<int64_t>& counts, const std::vector<int64_t>& w,
                           int G, int nb, float bin_size, std::vector<float>& corr) {
  // Space_Time_Correlation_Function::postprocess_list (space_time_correlation_function.cpp:345-360)
  corr.assign((size_t)G * nb, 0.f);
  for (int b = 0; b < nb; ++b) {
    const float rshell = b * bin_size;
    const float shellvolume =
        (float)((4.0 / 3.0) * PI_STCF * (std::pow(rshell + bin_size, 3.0) - std::pow(rshell, 3.0)));
    for (int g = 0; g < G; ++g) {
      float c = (float)counts[(size_t)g * nb + b];
      c /= ((float)w[g] * shellvolume);
      corr[(size_t)g * nb + b] = c;
    }
  }
}

void Van_Hove_Self::analyze(Trajectory_List* list) {
  DispOut o = disp(system, list->handle(), false, nullptr, nullptr, 1.f, n_bins_, max_value_);
  normalise_stcf(o.gs, o.pairs, system->n_timegaps(), n_bins_, bin_size_, corr_);
}

void Van_Hove_Self::write(const std::string& file) const {
  // Space_Time_Correlation_Function::write (space_time_correlation_function.cpp:240-271)
  std::ofstream out = open_out(file);
  const int G = system->n_timegaps();
  out << "Correlation data created by AMDAT v." << SEMVER << "\n";
  out << n_bins_ << " bins\n";
  out << G << " times\n\n";
  out << "\t";
  for (int b = 0; b < n_bins_; ++b) out << bin_size_ / 2 + float(b) * bin_size_ << "\t";
  out << "\n";
  for (int g = 0; g < G; ++g) {
    out << system->timegaps()[g] << "\t";
    for (int b = 0; b < n_bins_ - 1; ++b) out << Num{corr_[(size_t)g * n_bins_ + b]} << "\t";
    out << Num{corr_[(size_t)g * n_bins_ + n_bins_ - 1]} << "\n";
  }
}

// --- Gaussian comparison and fast particles ----------------------------------
namespace {
constexpr double GC_PI = 3.14159265;  // src/gaussian_comparison.cpp:15
}

Gaussian_Comparison::Gaussian_Comparison(System* sys, int time_index, const Van_Hove_Self& vhs, float msd)
    : sys_(sys), time_index_(time_index), n_bins_(vhs.show_n_bins()), bin_size_(vhs.show_bin_size()) {
  if (time_index < 0 || time_index >= sys->n_timegaps())
    throw Error(AMDAT_ERR_ARGUMENT, "time index of the Gaussian comparison out of range");
  // scale_van_hoves: both curves times the shell volume, the reference's
  // float/double mix (float storage, double pow/exp)
  const float alpha = (float)(3.0 / (2.0 * (double)msd));
  gaussian_.assign(n_bins_, 0.f);
  van_hove_.assign(n_bins_, 0.f);
  for (int b = 0; b < n_bins_; ++b) {
    const float inner = float(b) * bin_size_;
    const float shell = (float)(4.0 / 3.0 * GC_PI *
                                (std::pow(((double)float(b) + 1.0) * (double)bin_size_, 3.0) - std::pow((double)inner, 3.0)));
    van_hove_[b] = vhs.show(time_index, b) * shell;
    const double r = ((double)float(b) + .5) * (double)bin_size_;
    gaussian_[b] = (float)(std::pow((double)alpha / GC_PI, 3.0 / 2.0) * std::exp(-(double)alpha * std::pow(r, 2.0)) *
                           (double)shell);
  }
  // find_crossovers
  for (int b = 1; b < n_bins_; ++b)
    if (gaussian_[b] >= van_hove_[b]) {
      slow_index_ = b - 1;
      break;
    }
  for (int b = slow_index_ + 1; b < n_bins_; ++b)
    if (gaussian_[b] <= van_hove_[b]) {
      fast_index_ = b;
      break;
    }
  error_ = fast_index_ == 0;
  slowboundary_ = (float)std::pow(((double)float(slow_index_) + .5) * (double)bin_size_, 2.0);
  fastboundary_ = (float)std::pow(((double)float(fast_index_) - .5) * (double)bin_size_, 2.0);
  // determine_fractions
  for (int b = 1; b <= slow_index_; ++b) {
    slow_ += van_hove_[b];
    gslow_ += gaussian_[b];
  }
  fast_ = (float)(1.0 - (double)slow_);
  gfast_ = (float)(1.0 - (double)gslow_);
  for (int b = slow_index_ + 1; b < fast_index_; ++b) {
    fast_ -= van_hove_[b];
    gfast_ -= gaussian_[b];
  }
}

void Gaussian_Comparison::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  if (error_)
    out << "Warning: program cannot identify two crossing points between self Van Hove and Gaussian "
           "approximation self Van Hove.  Fractions of slow and fast particles will be incorrect.\n";
  out << "Gaussian comparison data created by AMDAT v." << SEMVER << "\n";
  out << "t*\n" << sys_->timegaps()[time_index_] << "\n";
  out << "Slow_Cutoff: " << std::pow((double)slowboundary_, 0.5) << "\n";
  out << "Fast_Cutoff: " << std::pow((double)fastboundary_, 0.5) << "\n";
  out << "\tSlow_Fraction\tFast_Fraction\n";
  out << "Gaussian\t" << gslow_ << "\t" << gfast_ << "\n";
  out << "Actual\t" << slow_ << "\t" << fast_ << "\n";
  out << "Excess\t" << slow_ - gslow_ << "\t" << fast_ - gfast_ << "\n\n";
  out << "Self_Van_Hove*shellvolume\n";
  out << "radius\tgaussian\tactual\n";
  for (int b = 0; b < n_bins_; ++b)
    out << (b + .5) * (double)bin_size_ << "\t" << Num{gaussian_[b]} << "\t" << Num{van_hove_[b]} << "\n";
}

std::unique_ptr<Trajectory_List> fast_particles(System* sys, Trajectory_List* list, int gap, float min_u2,
                                                std::vector<int64_t>* block_counts) {
  if (list->time_dependent())
    throw Error(AMDAT_ERR_ARGUMENT, "fast particles of a time-dependent list are not supported by this engine");
  if (gap < 0 || gap >= sys->n_timegaps()) throw Error(AMDAT_ERR_ARGUMENT, "time index out of range");
  int32_t h = 0;
  check(amdat_fast_particles(sys->ctx(), list->handle(), gap, min_u2, &h), "fast particles");
  auto bins = std::make_shared<Trajectory_List_Bins>(sys, h);
  if (block_counts) {
    std::vector<int64_t> per_frame((size_t)sys->n_timesteps(), 0);
    check(amdat_bins_read(sys->ctx(), h, AMDAT_OUT_HOST, nullptr, per_frame.data()), "fast particle counts");
    const int nb = sys->n_exponentials(), K = sys->n_exponential_steps();
    block_counts->assign(nb, 0);
    for (int b = 0; b < nb; ++b) {
      const int t = b * K + sys->show_frt();  // the block's first frame
      if (t >= 0 && t < sys->n_timesteps()) (*block_counts)[b] = per_frame[t];
    }
  }
  return std::make_unique<Trajectory_List>(sys, std::move(bins));
}

void write_block_counts(const System* sys, const std::vector<int64_t>& counts, const std::string& file) {
  // Exptime_Trajectory_List::write_count (src/exptime_trajectory_list.cpp)
  const int nb = (int)counts.size();
  double avg = 0;
  for (int b = 0; b < nb; ++b) avg += double(counts[b]) / double(nb);
  std::ofstream out = open_out(file);
  out << "Average_trajectories:\t" << avg << "\n";
  out << "Count_List\n";
  for (int b = 0; b < nb; ++b)
    out << sys->show_time(b * sys->n_exponential_steps() + sys->show_frt()) << "\t" << counts[b] << "\n";
}

Van_Hove_Distinct::Van_Hove_Distinct(System* sys, int n_bins, float max_value)
    : Van_Hove_Self(sys, n_bins, max_value) {}

void Van_Hove_Distinct::analyze(Trajectory_List* list) { analyze(list, list); }

void Van_Hove_Distinct::analyze(Trajectory_List* a, Trajectory_List* b) {
  const int G = system->n_timegaps();
  std::vector<int64_t> counts((size_t)G * n_bins_);
  check(amdat_vhd_run(system->ctx(), a->handle(), b->handle(), 0, max_value_, n_bins_,
                      AMDAT_OUT_HOST, counts.data()),
        "distinct van Hove run");
  // weighting: sum over time pairs of n1(t0) * n2 less the i == j pairs
  int64_t overlap = 0;
  {
    const auto& x = a->atoms();
    const auto& y = b->atoms();
    size_t i = 0, j = 0;
    while (i < x.size() && j < y.size()) {
      if (x[i] == y[j]) { ++overlap; ++i; ++j; }
      else if (x[i] < y[j]) ++i;
      else ++j;
    }
  }
  int64_t np = 0;
  int32_t T = 0, GG = 0;
  check(amdat_scheme_counts(&system->scheme(), 0, 0, &T, &GG, &np), "scheme");
  std::vector<int32_t> gap(np), t0(np), t1(np);
  check(amdat_scheme_pairs(&system->scheme(), 0, 0, gap.data(), t0.data(), t1.data()), "pairs");
  std::vector<int64_t> w(G, 0);
  for (int64_t p = 0; p < np; ++p)
    w[gap[p]] += (int64_t)a->show_n_trajectories() * b->show_n_trajectories() - overlap;
  normalise_stcf(counts, w, G, n_bins_, bin_size_, corr_);
}

// --- Fourier densities -------------------------------------------------------
Wave_Density::Wave_Density(System* sys, const Wave_Vectors* wv, int inner, int outer)
    : system_(sys), wv_(wv), first_(inner), last_(outer) {
  if (inner < 0 || outer >= wv->n_shells() || outer < inner)
    throw Error(AMDAT_ERR_ARGUMENT, "wavenumber index out of range");
}

Wave_Density::~Wave_Density() {
  if (handle_ >= 0) amdat_wave_density_free(system_->ctx(), handle_);
}

void Wave_Density::analyze(Trajectory_List* list) {
  std::vector<int32_t> kv, off;
  wv_->shells(first_, last_, kv, off);
  std::vector<int32_t> frames(system_->n_timesteps());
  for (int t = 0; t < (int)frames.size(); ++t) frames[t] = t;
  if (handle_ >= 0) amdat_wave_density_free(system_->ctx(), handle_);
  check(amdat_wave_density(system_->ctx(), list->handle(), kv.data(), (int32_t)kv.size() / 3,
                           wv_->period(), frames.data(), (int32_t)frames.size(), AMDAT_MIXED,
                           &handle_),
        "wave density");
  n_list_ = list->show_n_trajectories();
}

Intermediate_Scattering_Function::Intermediate_Scattering_Function(System* sys, Wave_Density* wd1,
                                                                   Wave_Density* wd2, int inner,
                                                                   int outer, bool fb)
    : system_(sys), wv_(wd1->wavevectors()), first_(inner), last_(outer) {
  if (wd1->wavevectors() != wd2->wavevectors())
    throw Error(AMDAT_ERR_ARGUMENT, "Wave vectors for density distributions do not match!");
  if (inner < wd1->first() || inner < wd2->first() || outer > wd1->last() || outer > wd2->last())
    throw Error(AMDAT_ERR_ARGUMENT, "requested wavenumber outside the Fourier density's range");
  const int G = sys->n_timegaps(), S = outer - inner + 1;
  // shells inner..outer inside the densities' vector list
  std::vector<int32_t> kv, off_all, off;
  wv_->shells(wd1->first(), wd1->last(), kv, off_all);
  for (int m = inner; m <= outer + 1; ++m) off.push_back(off_all[m - wd1->first()]);
  std::vector<double> corr((size_t)G * S);
  std::vector<int64_t> pc(G);
  check(amdat_isf_run(sys->ctx(), wd1->handle(), wd2->handle(), fb ? 1 : 0, off.data(), S,
                      AMDAT_OUT_HOST, corr.data(), pc.data()),
        "coherent ISF");
  // corr / (n_atoms * weighting) = corr / (pairs * N(t0)) (intermediate_scattering_function.cpp:312)
  corr_.assign((size_t)G * S, 0.f);
  for (int g = 0; g < G; ++g)
    for (int s = 0; s < S; ++s)
      corr_[(size_t)g * S + s] = (float)(corr[(size_t)g * S + s] / ((double)pc[g] * wd1->n_list()));
}

void Intermediate_Scattering_Function::write(const std::string& file) const {
  write_corr2d(file, system_, wv_, first_, last_, corr_);
}

// --- S(k) ------------------------------------------------------------------
Structure_Factor::Structure_Factor(System* sys, const Wave_Vectors* wv, int timescheme)
    : wv_(wv), timescheme_(timescheme) {
  system = sys;
}

void Structure_Factor::analyze(Trajectory_List* list) { analyze(list, list); }

void Structure_Factor::analyze(Trajectory_List* a, Trajectory_List* b) {
  std::vector<int32_t> kv, off;
  const int S = wv_->n_shells();
  wv_->shells(0, S - 1, kv, off);
  const std::vector<int32_t> frames = onetime_frames(*system, timescheme_);
  int32_t h1 = -1, h2 = -1;
  check(amdat_wave_density(system->ctx(), a->handle(), kv.data(), (int32_t)kv.size() / 3,
                           wv_->period(), frames.data(), (int32_t)frames.size(), AMDAT_MIXED, &h1),
        "wave density");
  if (b != a)
    check(amdat_wave_density(system->ctx(), b->handle(), kv.data(), (int32_t)kv.size() / 3,
                             wv_->period(), frames.data(), (int32_t)frames.size(), AMDAT_MIXED, &h2),
          "wave density");
  std::vector<double> s(S);
  const amdat_status st = amdat_structure_factor_run(system->ctx(), h1, b != a ? h2 : h1, off.data(),
                                                     S, AMDAT_OUT_HOST, s.data());
  amdat_wave_density_free(system->ctx(), h1);
  if (h2 >= 0) amdat_wave_density_free(system->ctx(), h2);
  check(st, "structure factor");
  // postprocess_list: S /= sum over frames of n(t) (structure_factor.cpp:272-285)
  const double n_total = (double)a->show_n_trajectories() * frames.size();
  sq_.assign(S, 0.f);
  for (int m = 0; m < S; ++m) sq_[m] = n_total != 0 ? (float)(s[m] / n_total) : 0.f;
}

void Structure_Factor::analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool) {
  if (list->time_dependent()) throw Error(AMDAT_ERR_ARGUMENT, "structure_factor bins take a static list here");
  std::vector<int32_t> kv, off;
  const int S = wv_->n_shells(), B = bins->n_bins();
  wv_->shells(0, S - 1, kv, off);
  const std::vector<int32_t> frames = onetime_frames(*system, timescheme_);
  std::vector<double> s((size_t)B * S);
  std::vector<int64_t> n(B);
  check(amdat_structure_factor_bins(system->ctx(), list->handle(), bins->handle(), kv.data(), (int32_t)kv.size() / 3,
                                    off.data(), S, wv_->period(), frames.data(), (int32_t)frames.size(), s.data(),
                                    n.data()),
        "binned structure factor");
  // postprocess_list per bin: S /= the members counted over the frames
  bin_sq_.assign(B, std::vector<float>(S, 0.f));
  for (int b = 0; b < B; ++b)
    for (int m = 0; m < S; ++m) bin_sq_[b][m] = n[b] != 0 ? (float)(s[(size_t)b * S + m] / (double)n[b]) : 0.f;
}

void Structure_Factor::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  out << "Structure factor data created by AMDAT v." << SEMVER << "\n";
  out << "Nominal_q\tMean_q\tStddev_q\tMean_qx\tMean_qy\tMean_qz\tS(q)\n";
  for (int m = 0; m < wv_->n_shells(); ++m) {
    const Coord mv = wv_->mean_wavevector(m);
    out << wv_->approx_wavenumber(m) << "\t" << wv_->mean_wavenumber(m) << "\t"
        << wv_->stdev_wavenumber(m) << "\t" << mv.x << "\t" << mv.y << "\t" << mv.z << "\t"
        << Num{sq_[m]} << std::endl;
  }
  out << "\n";
}

// --- RDF -------------------------------------------------------------------
Radial_Distribution_Function::Radial_Distribution_Function(System* sys, int n_bins, int timescheme,
                                                           float maxdistance)
    : n_bins_(n_bins), timescheme_(timescheme) {
  system = sys;
  if (n_bins < 1) throw Error(AMDAT_ERR_ARGUMENT, "need >= 1 bin");
  // constructor (radial_distribution_function.cpp:32-79)
  float minbox = sys->min_box();
  if (std::fabs(minbox - 1.0f) <= 1e-7f) {
    const Coord s = sys->size();
    minbox = std::min(s.x, s.y);
  }
  max_distance_ = (maxdistance > 0 && maxdistance < minbox / 2) ? maxdistance : minbox / 2;
  bin_size_ = max_distance_ / float(n_bins_);
}

void Radial_Distribution_Function::analyze(Trajectory_List* list) { analyze(list, list); }

void Radial_Distribution_Function::analyze(Trajectory_List* a, Trajectory_List* b) {
  const std::vector<int32_t> frames = onetime_frames(*system, timescheme_);
  const int F = (int)frames.size();
  std::vector<int64_t> counts((size_t)F * n_bins_);
  check(amdat_rdf_run(system->ctx(), a->handle(), b->handle(), frames.data(), F, max_distance_,
                      n_bins_, AMDAT_OUT_HOST, counts.data()),
        "rdf run");
  // postprocess_list (radial_distribution_function.cpp:256-285), FP32
  const Coord box = system->size();
  const float boxvolume = box.x * box.y * box.z;
  const int ni = a->show_n_trajectories(), nj = b->show_n_trajectories();
  mean_rdf_.assign(n_bins_, 0.f);
  n_atoms_j_.assign(F, nj);
  boxvolume_ = boxvolume;
  int n_i_total = 0;
  for (int f = 0; f < F; ++f) {
    const float rhoj = float(nj) / boxvolume;
    n_i_total += ni;
    for (int bi = 0; bi < n_bins_; ++bi) {
      const float rshell = float(bi) * bin_size_;
      const float shellvolume =
          (float)((4.0 / 3.0) * PI_RDF * (std::pow(rshell + bin_size_, 3.0) - std::pow(rshell, 3.0)));
      float t = (float)counts[(size_t)f * n_bins_ + bi];
      t /= (float(ni) * rhoj * shellvolume);
      mean_rdf_[bi] += t * float(ni);
    }
  }
  for (int bi = 0; bi < n_bins_; ++bi) mean_rdf_[bi] /= float(n_i_total);
}

void Radial_Distribution_Function::structure_factor(const std::string& file, int n_ks) const {
  // FP32 as the reference: mean density over the analysed frames, then the
  // sine transform of g(r) - 1 at bin centres
  const int n_times = (int)n_atoms_j_.size();
  float mean_rho = 0.f;
  for (int t = 0; t < n_times; ++t) mean_rho += float(n_atoms_j_[t]) / boxvolume_ / float(n_times);
  const float min_k = (float)(2. * PI_RDF / max_distance_);
  std::vector<float> klist(std::max(n_ks, 0)), sk(std::max(n_ks, 0));
  for (int k = 0; k < n_ks; ++k) {
    klist[k] = min_k * float(k + 1);
    float acc = 0.f;
    for (int b = 0; b < n_bins_; ++b) {
      const float rshell = (float)((float(b) + 0.5) * bin_size_);
      acc += (mean_rdf_[b] - 1) * rshell * std::sin(klist[k] * rshell) / klist[k] * bin_size_;
    }
    sk[k] = (float)(1. + 4. * PI_RDF * mean_rho * acc);
  }
  std::ofstream out = open_out(file);
  out << "Structure factor data calculated from g(r) created by AMDAT v." << SEMVER << "\n";
  for (int k = 0; k < n_ks; ++k) out << klist[k] << "\t";
  out << "\n";
  for (int k = 0; k < n_ks; ++k) out << Num{sk[k]} << "\t";
  out << "\n";
}

void Radial_Distribution_Function::write(const std::string& file) const {
  std::ofstream out = open_out(file);
  out << "Radial distribution function data created by AMDAT v." << SEMVER << "\n";
  for (int b = 0; b < n_bins_; ++b) out << float(b) * bin_size_ + bin_size_ / 2 << "\t";
  out << "\n";
  for (int b = 0; b < n_bins_; ++b) out << Num{mean_rdf_[b]} << "\t";
  out << "\n";
}

}  // namespace amdat_host
