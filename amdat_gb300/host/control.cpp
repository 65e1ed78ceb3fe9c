// Input-script interpreter for the hot-path commands of AMDAT's Control
// (src/control.cpp: system :191-240, create_list :1873, limit :1860, msd :2163,
// ngp :3345, isfs :3198, isf :3107, structure_factor :2655, rdf :2836,
// vhs :2517, vhd :2559, pathcheck :1136).  Command lines, their arguments and
// the "list <name>" target lines are read exactly as the reference reads
// them; output files are written by the analysis classes.  Failures are
// reported as an amdat_status with a message instead of exit().
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>

#include "amdat_host.h"

namespace amdat_host {

namespace {

class Control {
 public:
  explicit Control(int device) : device_(device) {}

  void run(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw Error(AMDAT_ERR_ARGUMENT, "input file " + path + " not found");
    std::string line;
    while (std::getline(in, line)) {
      const auto t = tokenize(line);
      if (t.empty() || t[0].find('#') != std::string::npos) continue;
      lines_.push_back(line);
    }
    while (pos_ < lines_.size()) {
      // tokens led by the flag marker '\\' are flags (Control::Control sets the
      // marker, src/control.cpp:161; Tokenize::parse_token): '\\sname' stores
      // the analysis under 'name'
      flags_.clear();
      std::vector<std::string> args;
      for (auto& tok : tokenize(lines_[pos_++])) {
        if (tok.size() >= 2 && tok[0] == '\\') flags_[tok[1]] = tok.substr(2);
        else args.push_back(tok);
      }
      if (!args.empty()) execute(args);
    }
  }

 private:
  std::string read_line() {
    if (pos_ >= lines_.size()) throw Error(AMDAT_ERR_ARGUMENT, "input script ended early");
    return lines_[pos_++];
  }

  static void pathcheck(const std::string& f) {
    const std::filesystem::path p(f);
    if (!std::filesystem::is_directory(p.parent_path()))
      throw Error(AMDAT_ERR_ARGUMENT, "Cannot write to filename.");
  }

  static void argcheck(const std::vector<std::string>& a, size_t lo, size_t hi) {
    if (a.size() < lo || a.size() > hi)
      throw Error(AMDAT_ERR_ARGUMENT, "Incorrect number of arguments for " + a[0] + ".");
  }

  System& sys() {
    if (!sys_) throw Error(AMDAT_ERR_STATE, "no system defined before " + lines_[pos_ - 1]);
    return *sys_;
  }

  Trajectory_List* list(const std::string& name) {
    auto it = lists_.find(name);
    if (it == lists_.end()) throw Error(AMDAT_ERR_ARGUMENT, "Trajectory list '" + name + "' not found.");
    return it->second.get();
  }

  // target line "list <name> [<name2>]"
  std::vector<Trajectory_List*> targets() {
    const auto a = tokenize(read_line());
    if (a.size() < 2 || a[0] != "list")
      throw Error(AMDAT_ERR_ARGUMENT, "only 'list <name>' targets are supported by this engine");
    std::vector<Trajectory_List*> out;
    for (size_t i = 1; i < a.size(); ++i) {
      out.push_back(list(a[i]));
      if (out.back()->time_dependent())
        throw Error(AMDAT_ERR_ARGUMENT, "time-dependent lists (find_fast) are supported by msd, msd_2d, mean_displacement, ngp and isfs here");
    }
    return out;
  }

  // Bin_Static_Analysis::write / Bin_Dynamics_Analysis::write file names: each
  // index goes through `ss << i; ss.seekp(0)` on one stringstream per axis, so
  // a shorter number overwrites only the front of a longer one written before
  static std::vector<std::string> bin_file_names(const std::string& stem, const Trajectory_List_Bins& b,
                                                 const char* sep) {
    auto put = [](std::string& buf, int v) {
      const std::string t = std::to_string(v);
      if (t.size() >= buf.size()) buf = t;
      else buf.replace(0, t.size(), t);
    };
    std::vector<std::string> out;
    std::string sx, sy, sz;
    for (int x = 0; x < b.show_n_xbins(); ++x)
      for (int y = 0; y < b.show_n_ybins(); ++y)
        for (int z = 0; z < b.show_n_zbins(); ++z) {
          put(sx, x), put(sy, y), put(sz, z);
          out.push_back(stem + "_bin_" + sx + sep + sy + sep + sz + ".bindata");
        }
    return out;
  }

  // target line "list <name> [<name2>]" or "bin_list <bins> <list> [persistence]"
  // (Control::run_analysis, src/control.h:268-380)
  // dynamic: a time-correlation analysis (Control sets `dynamic`), whose bin_list
  // target can take persistence (Bin_Dynamics_Analysis); static ones always run
  // Bin_Static_Analysis
  void analyze_write(Analysis& an, const std::string& file, bool dynamic = true) {
    const auto a = tokenize(read_line());
    if (!a.empty() && a[0] == "bin_list") {
      if (a.size() < 3) throw Error(AMDAT_ERR_ARGUMENT, "Insufficient number of arguments in bin_list target line.");
      auto it = bins_.find(a[1]);
      if (it == bins_.end()) throw Error(AMDAT_ERR_ARGUMENT, "Binned Trajectory list '" + a[1] + "' not found.");
      Trajectory_List* l = list(a[2]);
      const bool persistent = dynamic && a.size() >= 4 && std::atoi(a[3].c_str()) != 0;
      an.analyze_bins(l, it->second.get(), persistent);
      const auto names = bin_file_names(file, *it->second, persistent ? "." : "_");
      for (size_t b = 0; b < names.size(); ++b) {
        an.select_bin((int)b);
        an.write(names[b]);
      }
      return;
    }
    if (a.size() < 2 || a[0] != "list")
      throw Error(AMDAT_ERR_ARGUMENT, "Command " + (a.empty() ? std::string() : a[0]) +
                                          " not understood. Acceptable options are list or bin_list.");
    std::vector<Trajectory_List*> t;
    for (size_t i = 1; i < a.size(); ++i) t.push_back(list(a[i]));
    if (t.size() == 1 && t[0]->time_dependent()) {
      // a time-dependent list: its members at each start frame (one-bin static pass)
      an.analyze_bins(t[0], t[0]->membership(), false);
      an.select_bin(0);
      an.write(file);
      return;
    }
    for (auto* l : t)
      if (l->time_dependent())
        throw Error(AMDAT_ERR_ARGUMENT, "time-dependent lists (find_fast) are supported by msd, msd_2d, mean_displacement, ngp and isfs here");
    if (t.size() == 1) an.analyze(t[0]);
    else an.analyze(t[0], t[1]);
    an.write(file);
  }

  // Control::create_bin_list (src/control.cpp:3841-4000): "all nx ny nz" or
  // "region nx ny nz xlo xhi ylo yhi zlo zhi"
  void create_bin_list(const std::vector<std::string>& a) {
    argcheck(a, 2, 2);
    const auto s = tokenize(read_line());
    if (s.empty()) throw Error(AMDAT_ERR_ARGUMENT, "No set type found.");
    auto need = [&](size_t n) {
      if (s.size() != n)
        throw Error(AMDAT_ERR_ARGUMENT, "Incorrect number of arguments for command create_bin_list.");
    };
    auto i = [&](size_t k) { return std::atoi(s[k].c_str()); };
    auto f = [&](size_t k) { return (float)std::atof(s[k].c_str()); };
    std::unique_ptr<Trajectory_List_Bins> b;
    if (s[0] == "all") {
      need(4);
      b = std::make_unique<Trajectory_List_Bins>(&sys(), i(1), i(2), i(3));
    } else if (s[0] == "region") {
      need(10);
      b = std::make_unique<Trajectory_List_Bins>(&sys(), i(1), i(2), i(3), f(4), f(5), f(6), f(7), f(8), f(9));
    } else if (s[0] == "distance") {
      // distance trajectory <list> <from list> <thickness> <n_bins>
      // distance point <list> <x> <y> <z> <thickness> <n_bins>
      // distance plane <average|above|below> <list> <x|y|z> <position> <thickness> <n_bins>
      const std::string sub = s.size() > 1 ? s[1] : "";
      if (sub == "trajectory") {
        need(6);
        b = std::make_unique<Trajectory_List_Bins>(&sys(), f(4), i(5), list(s[2]), list(s[3]));
      } else if (sub == "point") {
        need(8);
        b = std::make_unique<Trajectory_List_Bins>(&sys(), f(6), i(7), list(s[2]), Coord{f(3), f(4), f(5)});
      } else if (sub == "plane") {
        need(8);
        b = std::make_unique<Trajectory_List_Bins>(&sys(), f(6), i(7), list(s[3]), s[4], f(5), s[2]);
      } else {
        throw Error(AMDAT_ERR_ARGUMENT,
                    "distance binning type " + sub + " not recognized, use trajectory, point or plane.");
      }
    } else {
      throw Error(AMDAT_ERR_ARGUMENT, "bin_list of type " + s[0] + " invalid");
    }
    bins_[a[1]] = std::move(b);
  }

  // selection commands of Analysis::analyze(string) (src/analysis.cpp:130-209)
  std::vector<int32_t> select(const std::vector<std::string>& a) {
    std::vector<int32_t> out;
    const auto& ty = sys().atom_types();
    const auto& sp = sys().atom_species();
    size_t i = 0;
    while (i < a.size()) {
      const std::string& c = a[i++];
      if (c == "all") {
        for (int k = 0; k < sys().n_atoms(); ++k) out.push_back(k);
      } else if (c == "type_system") {
        if (i >= a.size()) throw Error(AMDAT_ERR_ARGUMENT, "Insufficient arguments for type_system.");
        const int t = sys().atomtype_index(a[i++]);
        if (t < 0) throw Error(AMDAT_ERR_ARGUMENT, "atom type not found.");
        for (int k = 0; k < sys().n_atoms(); ++k)
          if (ty[k] == t) out.push_back(k);
      } else if (c == "species") {
        if (i >= a.size()) throw Error(AMDAT_ERR_ARGUMENT, "Insufficient arguments for species.");
        const int s = sys().species_index(a[i++]);
        if (s < 0) throw Error(AMDAT_ERR_ARGUMENT, "species not found.");
        for (int k = 0; k < sys().n_atoms(); ++k)
          if (sp[k] == s) out.push_back(k);
      } else if (c == "type_species") {
        if (i + 1 >= a.size()) throw Error(AMDAT_ERR_ARGUMENT, "Insufficient arguments for type_species.");
        const int s = sys().species_index(a[i++]);
        const int t = sys().atomtype_index(a[i++]);
        if (s < 0 || t < 0) throw Error(AMDAT_ERR_ARGUMENT, "species or atom type not found.");
        for (int k = 0; k < sys().n_atoms(); ++k)
          if (sp[k] == s && ty[k] == t) out.push_back(k);
      } else {
        throw Error(AMDAT_ERR_ARGUMENT, "Atom set command " + c + " for analysis not understood.");
      }
    }
    return out;
  }

  void execute(const std::vector<std::string>& a) {
    const std::string& cmd = a[0];
    if (cmd == "system" || cmd == "system_nv") {
      std::vector<std::string> block;
      for (int k = 0; k < 4; ++k) block.push_back(read_line());
      const size_t n_species = tokenize(block[3]).size() / 2;
      block.push_back(read_line());  // atom types
      for (size_t s = 0; s < n_species; ++s) block.push_back(read_line());
      const auto ty = tokenize(block[0]);
      if (!ty.empty() && ty[0] == "xyz")
        for (int k = 0; k < 2; ++k) block.push_back(read_line());  // box size, box bounds
      lists_.clear();
      bins_.clear();
      vhs_.reset();
      gc_.reset();
      sys_.reset();
      sys_ = std::make_unique<System>(block, device_);
    } else if (cmd == "limit") {
      argcheck(a, 2, 2);
      sys().set_limit(std::atoi(a[1].c_str()));
    } else if (cmd == "create_list") {
      argcheck(a, 2, 2);
      auto sel = select(tokenize(read_line()));
      lists_[a[1]] = std::make_unique<Trajectory_List>(&sys(), std::move(sel));
    } else if (cmd == "create_bin_list") {
      create_bin_list(a);
    } else if (cmd == "msd") {
      argcheck(a, 2, 2);
      pathcheck(a[1]);
      Mean_Square_Displacement m(&sys());
      analyze_write(m, a[1]);
    } else if (cmd == "msd_2d") {
      argcheck(a, 3, 3);
      Mean_Square_Displacement_2D m(&sys(), a[2]);
      analyze_write(m, a[1]);
    } else if (cmd == "mean_displacement") {
      argcheck(a, 2, 2);
      Mean_Displacement m(&sys());
      analyze_write(m, a[1]);
    } else if (cmd == "u2dist") {
      argcheck(a, 5, 5);
      DebyeWaller_Dist d(&sys(), std::atoi(a[2].c_str()), (float)std::atof(a[3].c_str()),
                         std::atoi(a[4].c_str()));
      analyze_write(d, a[1]);
    } else if (cmd == "displacement_dist") {
      argcheck(a, 6, 6);
      Displacement_Distribution d(&sys(), (float)std::atof(a[2].c_str()), std::atoi(a[3].c_str()),
                                  (float)std::atof(a[4].c_str()), std::atoi(a[5].c_str()));
      analyze_write(d, a[1]);
    } else if (cmd == "ngp") {
      argcheck(a, 2, 2);
      pathcheck(a[1]);
      Non_Gaussian_Parameter n(&sys());
      analyze_write(n, a[1]);
    } else if (cmd == "isfs") {
      argcheck(a, 6, 7);
      pathcheck(a[1]);
      Wave_Vectors wv(&sys(), a[4], (float)std::atof(a[5].c_str()));
      Incoherent_Scattering_Function f(&sys(), &wv, std::atoi(a[2].c_str()), std::atoi(a[3].c_str()),
                                       a.size() == 7 && std::atoi(a[6].c_str()) != 0);
      analyze_write(f, a[1]);
    } else if (cmd == "vhs") {
      argcheck(a, 4, 4);
      pathcheck(a[1]);
      auto v = std::make_unique<Van_Hove_Self>(&sys(), std::atoi(a[3].c_str()), (float)std::atof(a[2].c_str()));
      analyze_write(*v, a[1]);
      vhs_ = std::move(v);  // vhs_defined: compare_gaussian reads the last one
    } else if (cmd == "compare_gaussian") {
      // Control::compare_gaussian (src/control.cpp:3378-3422): MSD and NGP of the
      // target list, then the comparison at the NGP peak (or the given time index)
      if (!vhs_)
        throw Error(AMDAT_ERR_STATE,
                    "self van hove not yet defined.  Self van hove must be calculated prior to compare_gaussian "
                    "calculation.");
      if (a.size() != 2 && a.size() != 3)
        throw Error(AMDAT_ERR_ARGUMENT, "Incorrect number of arguments for gaussian comparison method.");
      auto t = targets();
      Mean_Square_Displacement m(&sys());
      m.analyze(t[0]);
      Non_Gaussian_Parameter n(&sys());
      n.analyze(t[0]);
      const int ti = a.size() == 3 ? std::atoi(a[2].c_str()) : n.max();
      if (ti < 0) throw Error(AMDAT_ERR_ARGUMENT, "the non-Gaussian parameter has no positive maximum");
      gc_ = std::make_unique<Gaussian_Comparison>(&sys(), ti, *vhs_, m.show(ti));
      gc_->write(a[1]);
    } else if (cmd == "find_fast" || cmd == "find_fast_fixedthreshold") {
      // Control::find_fast / find_fast_fixedthreshold (src/control.cpp:3430-3500)
      int gap;
      float threshold;
      if (cmd == "find_fast") {
        argcheck(a, 3, 3);
        if (!gc_)
          throw Error(AMDAT_ERR_STATE,
                      "A guassian comparison analysis myst be defined prior to calculating fast particle list.");
        gap = gc_->show_time_index();
        threshold = gc_->show_fastboundary();
      } else {
        argcheck(a, 5, 5);
        gap = std::atoi(a[3].c_str());
        threshold = (float)std::atof(a[4].c_str());
      }
      auto t = targets();
      std::vector<int64_t> counts;
      auto fast = fast_particles(&sys(), t[0], gap, threshold, &counts);
      write_block_counts(&sys(), counts, a[2]);
      lists_[a[1]] = std::move(fast);
    } else if (cmd == "vhd") {
      argcheck(a, 5, 5);
      pathcheck(a[1]);
      Van_Hove_Distinct v(&sys(), std::atoi(a[4].c_str()), (float)std::atof(a[3].c_str()));
      analyze_write(v, a[1]);
    } else if (cmd == "structure_factor") {
      argcheck(a, 6, 6);
      pathcheck(a[1]);
      Wave_Vectors wv(&sys(), a[3], (float)std::atof(a[4].c_str()));
      Structure_Factor s(&sys(), &wv, std::atoi(a[5].c_str()));
      if (pos_ < lines_.size() && tokenize(lines_[pos_]).size() > 0 && tokenize(lines_[pos_])[0] == "bin_list") {
        // Control::structure_factor (src/control.cpp:2730-2747): bins need the symmetric form
        if (a[2] != "symmetric") throw Error(AMDAT_ERR_ARGUMENT, "Binning currently only functions with symmetric S(k).");
        analyze_write(s, a[1], false);
        return;
      }
      auto t1 = targets();
      if (a[2] == "symmetric") s.analyze(t1[0]);
      else if (a[2] == "asymmetric") s.analyze(t1[0], targets()[0]);
      else throw Error(AMDAT_ERR_ARGUMENT, "structure factor symmetry must be symmetric or asymmetric");
      s.write(a[1]);
    } else if (cmd == "isf") {
      argcheck(a, 8, 8);
      if (a[2] != "auto") throw Error(AMDAT_ERR_ARGUMENT, "only the 'auto' isf method is supported");
      pathcheck(a[1]);
      Wave_Vectors wv(&sys(), a[4]);
      const int inner = std::atoi(a[6].c_str()), outer = std::atoi(a[7].c_str());
      Wave_Density wd1(&sys(), &wv, inner, outer);
      wd1.analyze(targets()[0]);
      if (a[3] == "symmetric") {
        Intermediate_Scattering_Function f(&sys(), &wd1, &wd1, inner, outer, std::atoi(a[5].c_str()) != 0);
        f.write(a[1]);
      } else if (a[3] == "asymmetric") {
        Wave_Density wd2(&sys(), &wv, inner, outer);
        wd2.analyze(targets()[0]);
        Intermediate_Scattering_Function f(&sys(), &wd1, &wd2, inner, outer, std::atoi(a[5].c_str()) != 0);
        f.write(a[1]);
      } else {
        throw Error(AMDAT_ERR_ARGUMENT, "isf symmetry must be symmetric or asymmetric");
      }
    } else if (cmd == "rdf") {
      argcheck(a, 6, 6);
      pathcheck(a[1]);
      auto r = std::make_unique<Radial_Distribution_Function>(&sys(), std::atoi(a[3].c_str()),
                                                              std::atoi(a[4].c_str()),
                                                              (float)std::atof(a[5].c_str()));
      auto t1 = targets();
      if (a[2] == "symmetric") r->analyze(t1[0]);
      else if (a[2] == "asymmetric") r->analyze(t1[0], targets()[0]);
      else throw Error(AMDAT_ERR_ARGUMENT, "rdf symmetry must be symmetric or asymmetric");
      r->write(a[1]);
      auto fs = flags_.find('s');
      if (fs != flags_.end()) {
        // Control::rdf stores a copy under the flagged name (src/control.cpp:2900-2913)
        if (stored_rdf_.count(fs->second))
          throw Error(AMDAT_ERR_ARGUMENT, "an analysis is already stored with name " + fs->second);
        stored_rdf_[fs->second] = std::move(r);
      }
    } else if (cmd == "structure_factor_from_rdf") {
      // Control::structure_factor_from_rdf (src/control.cpp:3073-3099)
      argcheck(a, 4, 4);
      auto it = stored_rdf_.find(a[3]);
      if (it == stored_rdf_.end())
        std::cerr << "\nWarning: no analysis stored with name " << a[3]
                  << ". Structure factor not calculated.\n";
      else
        it->second->structure_factor(a[1], std::atoi(a[2].c_str()));
    } else {
      throw Error(AMDAT_ERR_ARGUMENT, "command '" + cmd + "' is not part of this engine's hot path");
    }
  }

  int device_;
  std::map<char, std::string> flags_;
  std::map<std::string, std::unique_ptr<Radial_Distribution_Function>> stored_rdf_;
  std::vector<std::string> lines_;
  size_t pos_ = 0;
  std::unique_ptr<System> sys_;
  std::unique_ptr<Van_Hove_Self> vhs_;
  std::unique_ptr<Gaussian_Comparison> gc_;
  std::map<std::string, std::unique_ptr<Trajectory_List>> lists_;
  std::map<std::string, std::unique_ptr<Trajectory_List_Bins>> bins_;
};

}  // namespace

int run_script(const std::string& path, int device, std::string* error) {
  try {
    Control c(device);
    c.run(path);
    return AMDAT_OK;
  } catch (const Error& e) {
    if (error) *error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    if (error) *error = e.what();
    return AMDAT_ERR_ARGUMENT;
  }
}

}  // namespace amdat_host

static thread_local std::string g_script_error;

extern "C" amdat_status amdat_run_script(const char* input_path, int32_t device) {
  g_script_error.clear();
  if (!input_path) return AMDAT_ERR_ARGUMENT;
  const int s = amdat_host::run_script(input_path, device, &g_script_error);
  return (amdat_status)s;
}

extern "C" const char* amdat_script_error(void) { return g_script_error.c_str(); }
