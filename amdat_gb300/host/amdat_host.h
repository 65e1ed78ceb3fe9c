// Host-side mirror of AMDAT's analysis interface on top of the amdat_gb300
// C ABI.
//
// Class names, constructor arguments, the analyze / postprocess_list / write
// sequence and the output files follow the reference (src/analysis.h:62-135,
// src/control.h:270-390), so an input script written for AMDAT's hot commands
// runs unchanged.  The per-atom kernels are replaced by calls into the GPU
// engine; normalisation and file writing stay here, in the reference's own
// FP32 order where that decides printed digits (integer-count outputs).
// Errors throw amdat_host::Error (never exit()); the C entry point
// amdat_run_script turns them into a status code.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/amdat_gb300.h"

namespace amdat_host {

// version written in the output-file headers (the file formats are those of
// AMDAT 1.0.1)
extern const char* const SEMVER;

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void check(amdat_status s, const char* what);
std::vector<std::string> tokenize(const std::string& line);

struct Coord {
  float x, y, z;
};

// System::System + read_custom (src/system.cpp:55-220, 894-1360): the system
// block, the trajectory and the time scheme, uploaded to one GPU context.
class System {
 public:
  // block: the lines that follow "system" (trajectory type, file line, time
  // scheme, species line, atom type line, one count line per species; for the
  // xyz type also the box-size line and the box-bounds line, src/system.cpp:389-407)
  System(const std::vector<std::string>& block, int device);
  ~System();
  System(const System&) = delete;
  System& operator=(const System&) = delete;

  amdat_ctx* ctx() const { return ctx_; }
  const amdat_scheme& scheme() const { return scheme_; }
  void set_limit(int limit);  // Control::limit (src/control.cpp:1860)
  int n_atoms() const { return n_atoms_; }
  int n_timesteps() const { return n_timesteps_; }
  int n_timegaps() const { return n_timegaps_; }
  int n_exponentials() const { return scheme_.n_exponentials; }
  int n_exponential_steps() const { return scheme_.n_exponential_steps; }
  const std::vector<float>& timegaps() const { return gap_times_; }
  float show_time(int frame) const { return timelist_[frame]; }
  int show_frt() const { return scheme_.frt; }
  Coord size() const { return Coord{box_[0], box_[1], box_[2]}; }
  float min_box() const;  // min_box_dimensions().min()
  int atomtype_index(const std::string& name) const;
  int species_index(const std::string& name) const;
  // box_boundary (src/system.cpp): the bounds as read, constant over time
  const float* bounds_lo() const { return box_lo_; }
  const float* bounds_hi() const { return box_hi_; }
  const std::vector<int>& atom_types() const { return atom_type_; }
  const std::vector<int>& atom_species() const { return atom_species_; }

 private:
  void read_custom(const std::string& file, bool byid);
  void read_xyz(const std::string& file);
  void unwrap_from_wrapped();
  amdat_ctx* ctx_ = nullptr;
  amdat_scheme scheme_{};
  int n_atoms_ = 0, n_timesteps_ = 0, n_timegaps_ = 0;
  float box_[3] = {0, 0, 0}, box_lo_[3] = {0, 0, 0}, box_hi_[3] = {0, 0, 0};
  std::vector<float> timelist_, gap_times_;
  std::vector<std::string> species_names_, type_names_;
  std::vector<int> molecules_per_species_;
  std::vector<std::vector<int>> type_counts_;  // [species][type] atoms per molecule
  std::vector<int> atom_type_, atom_species_;
  std::vector<float> U_, W_;  // parsed coordinates until uploaded
};

// Static_Trajectory_List: membership fixed over time, ascending atom index
// (src/static_trajectory_list.cpp, src/trajectory_list.cpp:315-333)
class Trajectory_List_Bins;

class Trajectory_List {
 public:
  Trajectory_List(System* sys, std::vector<int32_t> atoms);
  // Exptime_Trajectory_List (src/exptime_trajectory_list.cpp): membership that
  // changes with the exponential block of the frame, held as a one-bin map of
  // the engine over all atoms (Fast_Particles makes these)
  Trajectory_List(System* sys, std::shared_ptr<Trajectory_List_Bins> membership);
  int handle() const { return handle_; }
  int show_n_trajectories(int = 0) const { return (int)atoms_.size(); }
  const std::vector<int32_t>& atoms() const { return atoms_; }
  bool time_dependent() const { return (bool)membership_; }
  Trajectory_List_Bins* membership() const { return membership_.get(); }

 private:
  int handle_ = 0;
  std::vector<int32_t> atoms_;
  std::shared_ptr<Trajectory_List_Bins> membership_;
};

// Wave_Vectors(System*, plane, max_length_scale) (src/wave_vectors.cpp:77-171,
// 430-480): 99 shells read from <prefix>.NNN files (NNN = shell + 2); the
// prefix comes from AMDAT_QVECTORS (the reference compiles it in as WV3D).
class Wave_Vectors {
 public:
  Wave_Vectors(System* sys, const std::string& plane, float max_length_scale = 0);
  int n_shells() const { return (int)offsets_.size() - 1; }
  float spacing() const { return spacing_; }
  float delta() const { return delta_; }
  float period() const { return period_; }  // L of k = 2 pi n / L
  float approx_wavenumber(int m) const { return approx_[m]; }
  int vectorcount(int m) const { return offsets_[m + 1] - offsets_[m]; }
  // integer lattice vectors and offsets of shells m0..m1
  void shells(int m0, int m1, std::vector<int32_t>& kvec, std::vector<int32_t>& off) const;
  float mean_wavenumber(int m) const;
  float stdev_wavenumber(int m) const;
  Coord mean_wavevector(int m) const;

 private:
  Coord vec(int i) const;
  float spacing_ = 0, delta_ = 0, period_ = 0;
  std::vector<float> approx_;
  std::vector<int32_t> n_;       // [3 * total]
  std::vector<int32_t> offsets_; // [99 + 1]
};

// Trajectory_List_Bins (src/trajectory_list_bins.cpp:207-394, 949-1096): a
// rectangular grid of bins over the box, or over a region of it (a bound of 0,
// or one beyond the box, is the box's own); membership per frame from the
// wrapped coordinates, which are boxified first (Control::create_bin_list).
class Trajectory_List_Bins {
 public:
  Trajectory_List_Bins(System* sys, int nx, int ny, int nz);
  Trajectory_List_Bins(System* sys, int nx, int ny, int nz, float xlo, float xhi, float ylo, float yhi,
                       float zlo, float zhi);
  // distance bin lists (create_bin_list distance ..., src/control.cpp:3915-3990;
  // src/trajectory_list_bins.cpp:461-948): the members of `binning` by their
  // distance to the nearest member of `clustered`, to a point, or to a plane
  // ("x"/"y"/"z" at `position`, direction "average", "above" or "below"), in
  // bins of `thickness`; at most the number of bins the box holds
  Trajectory_List_Bins(System* sys, float thickness, int n_bins, Trajectory_List* binning,
                       Trajectory_List* clustered);
  Trajectory_List_Bins(System* sys, float thickness, int n_bins, Trajectory_List* binning,
                       const std::string& plane, float position, const std::string& direction);
  Trajectory_List_Bins(System* sys, float thickness, int n_bins, Trajectory_List* binning, Coord point);
  // takes over a one-bin map the engine made (amdat_fast_particles)
  Trajectory_List_Bins(System* sys, int one_bin_handle);
  ~Trajectory_List_Bins();
  Trajectory_List_Bins(const Trajectory_List_Bins&) = delete;
  Trajectory_List_Bins& operator=(const Trajectory_List_Bins&) = delete;
  int handle() const { return handle_; }
  int show_n_xbins() const { return n_[0]; }
  int show_n_ybins() const { return n_[1]; }
  int show_n_zbins() const { return n_[2]; }
  int n_bins() const { return n_[0] * n_[1] * n_[2]; }

 private:
  void assign(const float lo[3], const float hi[3]);
  System* sys_;
  int n_[3];
  int handle_ = 0;
};

class Analysis {
 public:
  virtual ~Analysis() = default;
  virtual void analyze(Trajectory_List* list) = 0;
  virtual void analyze(Trajectory_List* a, Trajectory_List* b);
  virtual void write(const std::string& file) const = 0;
  // Bin_Static_Analysis (persistent = false) / Bin_Dynamics_Analysis
  // (persistent = true, src/bin_static_analysis.h, src/bin_dynamics_analysis.h):
  // one result per bin, all from one pass; select_bin(b) makes write() write bin b
  virtual void analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent);
  virtual void select_bin(int) {}

 protected:
  System* system = nullptr;
};

// Mean_Square_Displacement (src/mean_square_displacement.cpp:140-199)
class Mean_Square_Displacement : public Analysis {
 public:
  explicit Mean_Square_Displacement(System* sys);
  void analyze(Trajectory_List* list) override;
  void write(const std::string& file) const override;
  void analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) override;
  void select_bin(int b) override { msd_ = bin_msd_[b]; }
  float show(int g) const { return msd_[g]; }
  std::vector<double> sum_d4;  // kept for the NGP of the same pass

 private:
  std::vector<float> msd_;
  std::vector<double> weighting_;
  std::vector<std::vector<float>> bin_msd_;
};

// Non_Gaussian_Parameter (src/non_gaussian_parameter.cpp:96-174); the
// reference runs a separate MSD pass first (src/control.cpp:3345-3372), the
// engine computes both moments in one.
class Non_Gaussian_Parameter : public Analysis {
 public:
  explicit Non_Gaussian_Parameter(System* sys);
  void analyze(Trajectory_List* list) override;
  void write(const std::string& file) const override;
  void analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) override;
  void select_bin(int b) override { ngp_ = bin_ngp_[b]; }
  int max() const;

 private:
  std::vector<float> ngp_;
  std::vector<std::vector<float>> bin_ngp_;
};

// Incoherent_Scattering_Function (src/incoherent_scattering_function.cpp:176-299)
class Incoherent_Scattering_Function : public Analysis {
 public:
  Incoherent_Scattering_Function(System* sys, const Wave_Vectors* wv, int inner, int outer,
                                 bool fullblock);
  void analyze(Trajectory_List* list) override;
  void write(const std::string& file) const override;
  void analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) override;
  void select_bin(int b) override { corr_ = bin_corr_[b]; }

 private:
  const Wave_Vectors* wv_;
  int first_, last_;
  bool fullblock_;
  std::vector<float> corr_;  // [gap][shell]
  std::vector<std::vector<float>> bin_corr_;
};

// Mean_Square_Displacement_2D (src/mean_square_displacement_2d.cpp:79-199):
// msd in one plane ("xy", "xz" or "yz")
class Mean_Square_Displacement_2D : public Analysis {
 public:
  Mean_Square_Displacement_2D(System* sys, const std::string& plane);
  void analyze(Trajectory_List* list) override;
  void write(const std::string& file) const override;
  void analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) override;
  void select_bin(int b) override { msd_ = bin_msd_[b]; }

 private:
  std::string plane_;
  int a_ = 0, b_ = 1;  // axes of the plane
  std::vector<float> msd_;
  std::vector<std::vector<float>> bin_msd_;
};

// Mean_Displacement (src/mean_displacement.cpp:149-199): mean vector displacement
class Mean_Displacement : public Analysis {
 public:
  explicit Mean_Displacement(System* sys);
  void analyze(Trajectory_List* list) override;
  void write(const std::string& file) const override;
  void analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) override;
  void select_bin(int b) override { md_ = bin_md_[b]; }

 private:
  std::vector<float> md_;  // [gap][3]
  std::vector<std::vector<float>> bin_md_;
};

// DebyeWaller_Dist (src/debyewaller_dist.cpp:14-99, command u2dist): the
// distribution of |dr|^2 at one time gap, its mean and variance; bins+1 bins of
// maxvalue/bins, the top one collecting the overflow
class DebyeWaller_Dist : public Analysis {
 public:
  DebyeWaller_Dist(System* sys, int bins, float maxvalue, int time_index);
  void analyze(Trajectory_List* list) override;
  void write(const std::string& file) const override;

 protected:
  int n_bins_, time_index_;
  float binsize_, time_;
  float mean_ = 0.f, variance_ = 0.f;
  std::vector<float> dist_;
};

// Displacement_Distribution (src/displacement_distribution.cpp:17-141, command
// displacement_dist): the same statistics; the power is only printed, as in
// the reference (its kernel squares the displacement whatever the power)
class Displacement_Distribution : public DebyeWaller_Dist {
 public:
  Displacement_Distribution(System* sys, float power, int bins, float maxvalue, int time_index);
  void write(const std::string& file) const override;

 private:
  float power_;
};

// Van_Hove_Self (src/van_hove_self.cpp:45-103 + space_time_correlation_function.cpp)
class Van_Hove_Self : public Analysis {
 public:
  Van_Hove_Self(System* sys, int n_bins, float max_value);
  void analyze(Trajectory_List* list) override;
  void write(const std::string& file) const override;
  int show_n_bins() const { return n_bins_; }
  float show_bin_size() const { return bin_size_; }
  float show(int gap, int bin) const { return corr_[(size_t)gap * n_bins_ + bin]; }

 protected:
  int n_bins_;
  float max_value_, bin_size_;
  std::vector<float> corr_;  // [gap][bin]
};

// Gaussian_Comparison (src/gaussian_comparison.cpp): the self van Hove at one
// time gap against the Gaussian of the same MSD, both times the shell volume;
// their crossings bound the slow and fast particles, and the fractions follow
class Gaussian_Comparison {
 public:
  Gaussian_Comparison(System* sys, int time_index, const Van_Hove_Self& vhs, float msd);
  void write(const std::string& file) const;
  int show_time_index() const { return time_index_; }
  float show_fastboundary() const { return fastboundary_; }

 private:
  System* sys_;
  int time_index_, n_bins_;
  float bin_size_;
  std::vector<float> gaussian_, van_hove_;
  int slow_index_ = 0, fast_index_ = 0;
  float slowboundary_ = 0, fastboundary_ = 0;
  float slow_ = 0, fast_ = 0, gslow_ = 0, gfast_ = 0;
  bool error_ = false;
};

// Fast_Particles (src/fast_particles.cpp): the members of `list` whose squared
// displacement over time gap `gap` exceeds min_u2, per exponential block, as a
// time-dependent list; block_counts gets the members of each block
// (Exptime_Trajectory_List::write_count writes them, see write_block_counts)
std::unique_ptr<Trajectory_List> fast_particles(System* sys, Trajectory_List* list, int gap, float min_u2,
                                                std::vector<int64_t>* block_counts);
void write_block_counts(const System* sys, const std::vector<int64_t>& counts, const std::string& file);

// Van_Hove_Distinct with the distance the reference intends to bin
// (src/van_hove_distinct.cpp:159-213)
class Van_Hove_Distinct : public Van_Hove_Self {
 public:
  Van_Hove_Distinct(System* sys, int n_bins, float max_value);
  void analyze(Trajectory_List* list) override;
  void analyze(Trajectory_List* a, Trajectory_List* b) override;
};

// Wave_Density (src/wave_density.cpp): rho(k,t) kept on the GPU
class Wave_Density {
 public:
  Wave_Density(System* sys, const Wave_Vectors* wv, int inner, int outer);
  ~Wave_Density();
  void analyze(Trajectory_List* list);  // every frame of the trajectory
  int handle() const { return handle_; }
  int n_list() const { return n_list_; }
  const Wave_Vectors* wavevectors() const { return wv_; }
  int first() const { return first_; }
  int last() const { return last_; }

 private:
  System* system_;
  const Wave_Vectors* wv_;
  int first_, last_;
  int handle_ = -1;
  int n_list_ = 0;
};

// Intermediate_Scattering_Function coherent (src/intermediate_scattering_function.cpp:237-316)
class Intermediate_Scattering_Function {
 public:
  Intermediate_Scattering_Function(System* sys, Wave_Density* wd1, Wave_Density* wd2, int inner,
                                   int outer, bool fullblock);
  void write(const std::string& file) const;

 private:
  System* system_;
  const Wave_Vectors* wv_;
  int first_, last_;
  std::vector<float> corr_;
};

// Structure_Factor (src/structure_factor.cpp:201-344) over the frames of
// Analysis_Onetime's time scheme (src/analysis_onetime.cpp:22-50)
class Structure_Factor : public Analysis {
 public:
  Structure_Factor(System* sys, const Wave_Vectors* wv, int timescheme);
  void analyze(Trajectory_List* list) override;
  void analyze(Trajectory_List* a, Trajectory_List* b) override;
  void write(const std::string& file) const override;
  // Bin_Static_Analysis<Structure_Factor>: S(k) of the list members in each bin,
  // membership per frame (a static analysis: persistence does not apply)
  void analyze_bins(Trajectory_List* list, Trajectory_List_Bins* bins, bool persistent) override;
  void select_bin(int b) override { sq_ = bin_sq_[b]; }

 private:
  const Wave_Vectors* wv_;
  int timescheme_;
  std::vector<float> sq_;
  std::vector<std::vector<float>> bin_sq_;
};

// Radial_Distribution_Function (src/radial_distribution_function.cpp:32-350)
class Radial_Distribution_Function : public Analysis {
 public:
  Radial_Distribution_Function(System* sys, int n_bins, int timescheme, float max_distance);
  void analyze(Trajectory_List* list) override;
  void analyze(Trajectory_List* a, Trajectory_List* b) override;
  void write(const std::string& file) const override;
  // Radial_Distribution_Function::structure_factor (radial_distribution_function.cpp:379-434):
  // S(k) = 1 + 4 pi rho sum_r (g(r) - 1) r sin(k r) / k dr at k = (i+1) 2 pi / max_distance
  void structure_factor(const std::string& file, int n_ks) const;

 private:
  int n_bins_, timescheme_;
  float max_distance_, bin_size_;
  std::vector<float> mean_rdf_;
  std::vector<int> n_atoms_j_;  // per analysed frame
  float boxvolume_ = 0.f;
};

// frames visited by Analysis_Onetime::analyze (src/analysis_onetime.cpp:22-50)
std::vector<int32_t> onetime_frames(const System& sys, int timescheme);

// Control: runs an input script (src/control.cpp:108-530, hot-path commands)
int run_script(const std::string& path, int device, std::string* error);

}  // namespace amdat_host
