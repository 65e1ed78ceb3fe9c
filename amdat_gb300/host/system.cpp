// System, lists and wave vectors of the host mirror (see amdat_host.h).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <thread>

#include "amdat_host.h"

namespace amdat_host {

const char* const SEMVER = "1.0.1+gb300";

void check(amdat_status s, const char* what) {
  if (s != AMDAT_OK) throw Error((int)s, std::string(what) + ": " + amdat_last_error());
}

std::vector<std::string> tokenize(const std::string& line) {
  std::vector<std::string> out;
  std::istringstream is(line);
  std::string t;
  while (is >> t) out.push_back(t);
  return out;
}

static amdat_scheme parse_scheme(const std::vector<std::string>& a) {
  amdat_scheme s{};
  if (a.empty()) throw Error(AMDAT_ERR_ARGUMENT, "missing time scheme line");
  if (a[0] == "linear") {
    if (a.size() != 3) throw Error(AMDAT_ERR_ARGUMENT, "Incorrect number of arguments for linear time style.");
    check(amdat_scheme_init(&s, AMDAT_LINEAR, std::atoi(a[1].c_str()), 1, 1.0f, 0, 0,
                            (float)std::atof(a[2].c_str())), "linear scheme");
  } else if (a[0] == "exponential") {
    if (a.size() != 7) throw Error(AMDAT_ERR_ARGUMENT, "Incorrect number of arguments for exponential time style.");
    check(amdat_scheme_init(&s, AMDAT_EXPONENTIAL, std::atoi(a[1].c_str()), std::atoi(a[2].c_str()),
                            (float)std::atof(a[3].c_str()), std::atoi(a[4].c_str()),
                            std::atoi(a[5].c_str()), (float)std::atof(a[6].c_str())), "exponential scheme");
  } else if (a[0] == "snapshot") {
    check(amdat_scheme_init(&s, AMDAT_SNAPSHOT, 1, 0, 1.0f, 0, 0, 1.0f), "snapshot scheme");
  } else {
    throw Error(AMDAT_ERR_ARGUMENT, "Time scheme " + a[0] + " not recognized!");
  }
  return s;
}

System::System(const std::vector<std::string>& block, int device) {
  // block: type / file line / time scheme / species / types / counts x species
  if (block.size() < 5) throw Error(AMDAT_ERR_ARGUMENT, "incomplete system block");
  const auto type = tokenize(block[0]);
  if (type.empty() || (type[0] != "custom" && type[0] != "custom_byid" && type[0] != "xyz"))
    throw Error(AMDAT_ERR_ARGUMENT,
                "only the custom, custom_byid and xyz trajectory types are supported by this engine");
  const bool xyz = type[0] == "xyz";
  const auto fileline = tokenize(block[1]);
  if (fileline.empty()) throw Error(AMDAT_ERR_ARGUMENT, "missing trajectory file");
  scheme_ = parse_scheme(tokenize(block[2]));
  int64_t npairs = 0;
  check(amdat_scheme_counts(&scheme_, 0, 0, &n_timesteps_, &n_timegaps_, &npairs), "scheme");
  timelist_.resize(n_timesteps_);
  gap_times_.resize(n_timegaps_);
  check(amdat_scheme_times(&scheme_, timelist_.data(), gap_times_.data()), "scheme times");
  const auto sp = tokenize(block[3]);
  if (sp.size() < 2 || sp.size() % 2) throw Error(AMDAT_ERR_ARGUMENT, "bad species line");
  for (size_t i = 0; i + 1 < sp.size(); i += 2) {
    species_names_.push_back(sp[i]);
    molecules_per_species_.push_back(std::atoi(sp[i + 1].c_str()));
  }
  type_names_ = tokenize(block[4]);
  if (block.size() < 5 + species_names_.size())
    throw Error(AMDAT_ERR_ARGUMENT, "missing atom count lines");
  for (size_t s = 0; s < species_names_.size(); ++s) {
    const auto c = tokenize(block[5 + s]);
    if (c.size() != type_names_.size()) {
      std::ostringstream m;
      m << "Number of atom counts (" << c.size() << ") does not match number of atom types("
        << type_names_.size() << ").";
      throw Error(AMDAT_ERR_ARGUMENT, m.str());
    }
    std::vector<int> v;
    for (auto& x : c) v.push_back(std::atoi(x.c_str()));
    type_counts_.push_back(v);
  }
  if (xyz) {
    // System::xyz_prep (src/system.cpp:389-407): "Lx Ly Lz", then
    // "xlo xhi ylo yhi zlo zhi", constant over the trajectory
    const size_t b = 5 + species_names_.size();
    if (block.size() < b + 2) throw Error(AMDAT_ERR_ARGUMENT, "missing box lines for the xyz trajectory");
    const auto L = tokenize(block[b]), lohi = tokenize(block[b + 1]);
    if (L.size() < 3 || lohi.size() < 6) throw Error(AMDAT_ERR_ARGUMENT, "bad box lines for the xyz trajectory");
    for (int d = 0; d < 3; ++d) {
      box_[d] = (float)std::atof(L[d].c_str());
      box_lo_[d] = (float)std::atof(lohi[2 * d].c_str());
      box_hi_[d] = (float)std::atof(lohi[2 * d + 1].c_str());
    }
  }
  n_atoms_ = 0;
  for (size_t s = 0; s < species_names_.size(); ++s) {
    int per = 0;
    for (int v : type_counts_[s]) per += v;
    for (int m = 0; m < molecules_per_species_[s]; ++m)
      for (int a = 0; a < per; ++a) atom_species_.push_back((int)s);
    n_atoms_ += molecules_per_species_[s] * per;
  }
  if (n_atoms_ <= 0) throw Error(AMDAT_ERR_ARGUMENT, "system has no atoms");
  // parse the whole trajectory before touching the GPU, so input errors are
  // reported the same way with or without a device
  if (xyz)
    read_xyz(fileline[0]);
  else
    read_custom(fileline[0], type[0] == "custom_byid");
  check(amdat_create(device, &ctx_), "amdat_create");
  try {
    check(amdat_traj_upload(ctx_, n_timesteps_, n_atoms_, U_.data(), W_.empty() ? nullptr : W_.data(),
                            box_, box_lo_),
          "trajectory upload");
    check(amdat_set_scheme(ctx_, &scheme_), "amdat_set_scheme");
  } catch (...) {
    amdat_destroy(ctx_);
    ctx_ = nullptr;
    throw;
  }
  std::vector<float>().swap(U_);
  std::vector<float>().swap(W_);
}

System::~System() {
  if (ctx_) amdat_destroy(ctx_);
}

void System::set_limit(int limit) {
  scheme_.limit = limit;
  check(amdat_set_scheme(ctx_, &scheme_), "limit");
}

float System::min_box() const { return std::min(box_[0], std::min(box_[1], box_[2])); }

int System::atomtype_index(const std::string& name) const {
  for (size_t i = 0; i < type_names_.size(); ++i)
    if (type_names_[i] == name) return (int)i;
  return -1;
}

int System::species_index(const std::string& name) const {
  for (size_t i = 0; i < species_names_.size(); ++i)
    if (species_names_[i] == name) return (int)i;
  return -1;
}

// --- LAMMPS custom dump reader ---------------------------------------------
namespace {

struct Cols {
  int x = -1, y = -1, z = -1, xs = -1, ys = -1, zs = -1, xu = -1, yu = -1, zu = -1;
  int xsu = -1, ysu = -1, zsu = -1, ix = -1, iy = -1, iz = -1, type = -1, id = -1;
};

// next line [p, eol) of a buffer; returns pointer after the line end
inline const char* next_line(const char* p, const char* end, const char** eol) {
  const char* e = (const char*)std::memchr(p, '\n', end - p);
  if (!e) e = end;
  *eol = e;
  return e < end ? e + 1 : end;
}

inline const char* field(const char* p, const char* eol, int k, const char** fend) {
  for (int i = 0;; ++i) {
    while (p < eol && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    const char* s = p;
    while (p < eol && *p != ' ' && *p != '\t' && *p != '\r') ++p;
    if (i == k) {
      *fend = p;
      return s;
    }
    if (p >= eol) {
      *fend = s;
      return s;
    }
  }
}

// the reference reads coordinates with atof (double) into float
inline float atof32(const char* s) { return (float)std::strtod(s, nullptr); }
inline double atof64(const char* s) { return std::strtod(s, nullptr); }

}  // namespace

// custom (src/system.cpp:1026-1360): atom lines in file order, grouped by species.
// custom_byid (src/system.cpp:2438-2936): atom lines in any order; the "id"
// column places each at index id-1 (ids must be 1..N), and an id keeps the type
// it had in the first frame.
void System::read_custom(const std::string& file, bool byid) {
  std::ifstream in(file, std::ios::binary);
  if (!in) throw Error(AMDAT_ERR_ARGUMENT, "Custom Trajectory file not found.");
  in.seekg(0, std::ios::end);
  const size_t size = (size_t)in.tellg();
  in.seekg(0);
  std::string buf(size, '\0');
  in.read(&buf[0], (std::streamsize)size);
  const char* p = buf.data();
  const char* end = p + size;
  const int T = n_timesteps_, N = n_atoms_;
  // locate each frame: header of 9 lines, then N atom lines
  std::vector<const char*> frame(T);
  Cols c;
  std::vector<std::string> colnames;
  for (int t = 0; t < T; ++t) {
    if (p >= end) throw Error(AMDAT_ERR_ARGUMENT, "trajectory file ends before frame " + std::to_string(t));
    frame[t] = p;
    const char* eol;
    for (int l = 0; l < 3; ++l) p = next_line(p, end, &eol);
    const int n = std::atoi(std::string(p, next_line(p, end, &eol) - p).c_str());
    p = next_line(p, end, &eol);
    if (n != N) {
      std::ostringstream m;
      m << "The number of atoms listed in the xyz file is inconsistent with user input: " << n
        << " != " << N;
      throw Error(AMDAT_ERR_ARGUMENT, m.str());
    }
    p = next_line(p, end, &eol);  // ITEM: BOX BOUNDS
    float lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      const char* s = p;
      p = next_line(p, end, &eol);
      const auto a = tokenize(std::string(s, eol));
      if (a.size() < 2) throw Error(AMDAT_ERR_ARGUMENT, "bad box bounds line");
      lo[d] = atof32(a[0].c_str());
      hi[d] = atof32(a[1].c_str());
    }
    if (t == 0) {
      for (int d = 0; d < 3; ++d) {
        box_lo_[d] = lo[d];
        box_hi_[d] = hi[d];
        box_[d] = hi[d] - lo[d];
      }
    } else {
      // constant volume (System::floatCompare, src/system.cpp:1002)
      for (int d = 0; d < 3; ++d) {
        const float a = box_lo_[d], b = lo[d], a2 = box_lo_[d] + box_[d], b2 = hi[d];
        auto same = [](float A, float B) {
          const float diff = std::fabs(A - B), L = std::max(std::fabs(A), std::fabs(B));
          return diff <= L * FLT_EPSILON;
        };
        if (!same(a, b) || !same(a2, b2))
          throw Error(AMDAT_ERR_ARGUMENT,
                      "The box boundaries provided in the custom file are not constant.");
      }
    }
    const char* s = p;
    p = next_line(p, end, &eol);  // ITEM: ATOMS ...
    if (t == 0) {
      colnames = tokenize(std::string(s, eol));
      auto find = [&](const char* nm) {
        for (size_t i = 2; i < colnames.size(); ++i)
          if (colnames[i] == nm) return (int)i - 2;
        return -1;
      };
      c.x = find("x"); c.y = find("y"); c.z = find("z");
      c.xs = find("xs"); c.ys = find("ys"); c.zs = find("zs");
      c.xu = find("xu"); c.yu = find("yu"); c.zu = find("zu");
      c.xsu = find("xsu"); c.ysu = find("ysu"); c.zsu = find("zsu");
      c.ix = find("ix"); c.iy = find("iy"); c.iz = find("iz");
      c.type = find("type");
      c.id = find("id");
      if (byid && c.id < 0) throw Error(AMDAT_ERR_ARGUMENT, "atom id data not provided.");
      if (c.type < 0) throw Error(AMDAT_ERR_ARGUMENT, "atom type data not provided.");
    }
    for (int a = 0; a < N; ++a) p = next_line(p, end, &eol);
  }
  const bool r = c.x >= 0 && c.y >= 0 && c.z >= 0, rs = c.xs >= 0 && c.ys >= 0 && c.zs >= 0;
  const bool ru = c.xu >= 0 && c.yu >= 0 && c.zu >= 0, rsu = c.xsu >= 0 && c.ysu >= 0 && c.zsu >= 0;
  const bool img = c.ix >= 0 && c.iy >= 0 && c.iz >= 0;
  if (!r && !rs && !ru && !rsu)
    throw Error(AMDAT_ERR_ARGUMENT, "No complete set of coordinates provided in trajectory file.");
  const bool read_i = !ru && !rsu && img && (r || rs);
  const bool have_w = r || rs;
  const bool have_u = ru || rsu || read_i;
  std::vector<float>& U = U_;
  std::vector<float>& W = W_;
  U.assign((size_t)T * N * 3, 0.f);
  W.assign(have_w ? (size_t)T * N * 3 : 0, 0.f);
  atom_type_.assign(N, 0);
  std::string bad_type;
  std::vector<int> bad_id(T, 0);           // 1: id out of 1..N or repeated, 2: type changed
  std::vector<unsigned char> seen(byid ? N : 0, 0);
  auto parse = [&](int t0, int t1) {
    for (int t = t0; t < t1; ++t) {
      const char* q = frame[t];
      const char* eol;
      for (int l = 0; l < 9; ++l) q = next_line(q, end, &eol);
      for (int line = 0; line < N; ++line) {
        const char* ls = q;
        q = next_line(q, end, &eol);
        const char* fe;
        int a = line;
        if (byid) {
          const char* is = field(ls, eol, c.id, &fe);
          a = std::atoi(std::string(is, fe).c_str()) - 1;
          if (a < 0 || a >= N) {
            bad_id[t] = 1;
            continue;
          }
          if (t == 0) {
            if (seen[a]) bad_id[t] = 1;
            seen[a] = 1;
          }
        }
        float* u = &U[((size_t)t * N + a) * 3];
        float* w = have_w ? &W[((size_t)t * N + a) * 3] : nullptr;
        if (t == 0 || byid) {
          const char* ts = field(ls, eol, c.type, &fe);
          const std::string tn(ts, fe);
          int ti = -1;
          for (size_t i = 0; i < type_names_.size(); ++i)
            if (type_names_[i] == tn) ti = (int)i;
          if (ti < 0 && t == 0) bad_type = tn;  // frame 0 is parsed alone
          if (t == 0)
            atom_type_[a] = ti < 0 ? 0 : ti;
          else if (ti < 0)
            bad_id[t] = 2;
          else if (ti >= 0 && ti != atom_type_[a])
            bad_id[t] = 2;
        }
        const int wx[3] = {c.x, c.y, c.z}, sx[3] = {c.xs, c.ys, c.zs};
        const int ux[3] = {c.xu, c.yu, c.zu}, sux[3] = {c.xsu, c.ysu, c.zsu};
        const int ix[3] = {c.ix, c.iy, c.iz};
        for (int d = 0; d < 3; ++d) {
          float wv = 0.f;
          if (r) wv = atof32(field(ls, eol, wx[d], &fe));
          else if (rs) wv = (float)((double)box_[d] * atof64(field(ls, eol, sx[d], &fe)) + (double)box_lo_[d]);
          if (w) w[d] = wv;
          if (read_i) u[d] = (float)((double)wv + atof64(field(ls, eol, ix[d], &fe)) * (double)box_[d]);
          else if (ru) u[d] = atof32(field(ls, eol, ux[d], &fe));
          else if (rsu) u[d] = (float)((double)box_[d] * atof64(field(ls, eol, sux[d], &fe)) + (double)box_lo_[d]);
          else u[d] = wv;
        }
      }
    }
  };
  // frame 0 first: it fixes each atom's type (and, by id, its index)
  parse(0, 1);
  if (T > 1) {
    const int nth = std::max(1, std::min<int>(T - 1, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int i = 0; i < nth; ++i)
      th.emplace_back(parse, 1 + (int)((int64_t)(T - 1) * i / nth), 1 + (int)((int64_t)(T - 1) * (i + 1) / nth));
    for (auto& x : th) x.join();
  }
  if (!bad_type.empty()) throw Error(AMDAT_ERR_ARGUMENT, "Atom type " + bad_type + " in trajectory file out of range!");
  for (int t = 0; t < T; ++t) {
    if (bad_id[t] == 1)
      throw Error(AMDAT_ERR_ARGUMENT,
                  "Some problem with handling atom ids during file read in. Atom ids should begin with 1 "
                  "and should not skip.");
    if (bad_id[t] == 2)
      throw Error(AMDAT_ERR_ARGUMENT, "Type of index in file does not match type in id map (frame " +
                                          std::to_string(t) + ").");
  }
  if (!have_u) unwrap_from_wrapped();
}

// Trajectory::unwrap (src/trajectory.cpp:236-271): unwrapped(0) = wrapped(0), then
// the step-to-step displacement corrected by L * int(d / (0.55 L)), in FP32
void System::unwrap_from_wrapped() {
  const int T = n_timesteps_, N = n_atoms_;
  std::vector<float>& U = U_;
  const std::vector<float>& W = W_;
  for (int a = 0; a < N; ++a)
    for (int t = 1; t < T; ++t)
      for (int d = 0; d < 3; ++d) {
        const float disp = W[((size_t)t * N + a) * 3 + d] - W[((size_t)(t - 1) * N + a) * 3 + d];
        const float den = box_[d] * 0.55f;
        const float q = (float)(int)(disp / den);
        const float corr = box_[d] * q;
        U[((size_t)t * N + a) * 3 + d] = U[((size_t)(t - 1) * N + a) * 3 + d] + (disp - corr);
      }
}

// System::read_xyz (src/system.cpp:610-700): per frame a line with the atom
// count, one comment line, then one "type x y z" line per atom in species and
// molecule order. Coordinates are wrapped and read straight into float; the
// type is its integer label (1-based). Unwrapped coordinates are derived.
void System::read_xyz(const std::string& file) {
  std::ifstream in(file, std::ios::binary);
  if (!in) throw Error(AMDAT_ERR_ARGUMENT, "XYZ Trajectory file not found.");
  in.seekg(0, std::ios::end);
  const size_t size = (size_t)in.tellg();
  in.seekg(0);
  std::string buf(size, '\0');
  in.read(&buf[0], (std::streamsize)size);
  const char* p = buf.data();
  const char* end = p + size;
  const int T = n_timesteps_, N = n_atoms_;
  std::vector<const char*> frame(T);
  for (int t = 0; t < T; ++t) {
    const char* eol;
    while (p < end && (*p == '\n' || *p == '\r' || *p == ' ' || *p == '\t')) ++p;
    if (p >= end) throw Error(AMDAT_ERR_ARGUMENT, "trajectory file ends before frame " + std::to_string(t));
    const char* s = p;
    p = next_line(p, end, &eol);
    const int n = std::atoi(std::string(s, eol).c_str());
    if (n != N) {
      std::ostringstream m;
      m << "The number of atoms listed in the xyz file is inconsistent with user input: " << n
        << " != " << N;
      throw Error(AMDAT_ERR_ARGUMENT, m.str());
    }
    p = next_line(p, end, &eol);  // comment line ("Atoms. Timestep: ...")
    frame[t] = p;
    for (int a = 0; a < N; ++a) {
      if (p >= end) throw Error(AMDAT_ERR_ARGUMENT, "trajectory file ends inside frame " + std::to_string(t));
      p = next_line(p, end, &eol);
    }
  }
  U_.assign((size_t)T * N * 3, 0.f);
  W_.assign((size_t)T * N * 3, 0.f);
  atom_type_.assign(N, 0);
  const int n_types = (int)type_names_.size();
  std::vector<int> bad(T, 0);
  auto parse = [&](int t0, int t1) {
    for (int t = t0; t < t1; ++t) {
      const char* q = frame[t];
      for (int a = 0; a < N; ++a) {
        const char* eol;
        const char* ls = q;
        q = next_line(q, end, &eol);
        const char* fe;
        const char* ts = field(ls, eol, 0, &fe);
        const int ty = std::atoi(std::string(ts, fe).c_str());
        if (ty < 1 || ty > n_types) bad[t] = 1;
        if (t == 0) atom_type_[a] = ty >= 1 && ty <= n_types ? ty - 1 : 0;
        float* w = &W_[((size_t)t * N + a) * 3];
        for (int d = 0; d < 3; ++d) {
          const char* xs = field(ls, eol, 1 + d, &fe);
          if (xs == fe) bad[t] = 2;
          w[d] = std::strtof(xs, nullptr);
        }
      }
    }
  };
  const int nth = std::max(1, std::min<int>(T, (int)std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int i = 0; i < nth; ++i) th.emplace_back(parse, (int)((int64_t)T * i / nth), (int)((int64_t)T * (i + 1) / nth));
  for (auto& x : th) x.join();
  for (int t = 0; t < T; ++t) {
    if (bad[t] == 1) throw Error(AMDAT_ERR_ARGUMENT, "Atom type in trajectory file out of range!");
    if (bad[t] == 2) throw Error(AMDAT_ERR_ARGUMENT, "incomplete atom line in xyz frame " + std::to_string(t));
  }
  // unwrapped(0) = wrapped(0)
  std::copy(W_.begin(), W_.begin() + (size_t)N * 3, U_.begin());
  unwrap_from_wrapped();
}

// --- lists -----------------------------------------------------------------
Trajectory_List::Trajectory_List(System* sys, std::vector<int32_t> atoms) : atoms_(std::move(atoms)) {
  std::sort(atoms_.begin(), atoms_.end());
  atoms_.erase(std::unique(atoms_.begin(), atoms_.end()), atoms_.end());
  if ((int)atoms_.size() == sys->n_atoms())
    handle_ = 0;
  else
    check(amdat_list_create(sys->ctx(), atoms_.data(), (int32_t)atoms_.size(), &handle_), "list");
}

Trajectory_List::Trajectory_List(System* sys, std::shared_ptr<Trajectory_List_Bins> membership)
    : handle_(0), membership_(std::move(membership)) {
  // the binned pass runs over all atoms and keys each by the membership map
  atoms_.resize(sys->n_atoms());
  for (int a = 0; a < sys->n_atoms(); ++a) atoms_[a] = a;
}

// --- wave vectors ----------------------------------------------------------
static const double PI_WV = 3.14159265358979323846;  // src/wave_vectors.cpp:16

Wave_Vectors::Wave_Vectors(System* sys, const std::string& plane, float max_length_scale) {
  if (plane != "xyz")
    throw Error(AMDAT_ERR_ARGUMENT, "only the xyz wave-vector plane is supported by this engine");
  const float min_size = max_length_scale <= 0.0f ? sys->min_box() : max_length_scale;
  spacing_ = (float)(2.0 * PI_WV / min_size);
  delta_ = (float)(spacing_ / 2.0);
  period_ = min_size;
  for (int m = 0; m < 99; ++m) approx_.push_back(spacing_ + delta_ * (float)m);
  const char* prefix = std::getenv("AMDAT_QVECTORS");
  if (!prefix || !*prefix)
    throw Error(AMDAT_ERR_ARGUMENT,
                "set AMDAT_QVECTORS to the q-vector file prefix (.../qvectors3d/qvector)");
  offsets_.push_back(0);
  for (int m = 0; m < 99; ++m) {
    char stem[16];
    std::snprintf(stem, sizeof(stem), ".%03d", m + 2);
    const std::string fn = std::string(prefix) + stem;
    std::ifstream f(fn);
    if (!f.is_open()) throw Error(AMDAT_ERR_ARGUMENT, "Error opening vector file" + fn);
    double x, y, z;
    while (f >> x >> y >> z) {
      n_.push_back((int32_t)std::lround(x));
      n_.push_back((int32_t)std::lround(y));
      n_.push_back((int32_t)std::lround(z));
    }
    offsets_.push_back((int32_t)(n_.size() / 3));
  }
}

void Wave_Vectors::shells(int m0, int m1, std::vector<int32_t>& kvec, std::vector<int32_t>& off) const {
  if (m0 < 0 || m1 >= n_shells() || m1 < m0) throw Error(AMDAT_ERR_ARGUMENT, "wavenumber index out of range");
  kvec.assign(n_.begin() + 3 * offsets_[m0], n_.begin() + 3 * offsets_[m1 + 1]);
  off.clear();
  for (int m = m0; m <= m1 + 1; ++m) off.push_back(offsets_[m] - offsets_[m0]);
}

Coord Wave_Vectors::vec(int i) const {
  return Coord{(float)n_[3 * i] * spacing_, (float)n_[3 * i + 1] * spacing_, (float)n_[3 * i + 2] * spacing_};
}

static float length32(const Coord& v) {
  const float xx = v.x * v.x, yy = v.y * v.y, zz = v.z * v.z;
  return std::sqrt((xx + yy) + zz);
}

// show_mean_wavenumber / show_stdev_wavenumber / show_mean_wavevector
// (src/wave_vectors.cpp:527-566), FP32 as in the reference
float Wave_Vectors::mean_wavenumber(int m) const {
  float s = 0;
  for (int i = offsets_[m]; i < offsets_[m + 1]; ++i) s += length32(vec(i));
  return s / (float)vectorcount(m);
}

float Wave_Vectors::stdev_wavenumber(int m) const {
  const float mean = mean_wavenumber(m);
  float var = 0;
  for (int i = offsets_[m]; i < offsets_[m + 1]; ++i)
    var = (float)((double)var + std::pow((double)(length32(vec(i)) - mean), 2.0));
  var /= (float)vectorcount(m);
  return (float)std::pow((double)var, 0.5);
}

Coord Wave_Vectors::mean_wavevector(int m) const {
  Coord s{0, 0, 0};
  for (int i = offsets_[m]; i < offsets_[m + 1]; ++i) {
    const Coord v = vec(i);
    s.x += v.x;
    s.y += v.y;
    s.z += v.z;
  }
  const float n = (float)vectorcount(m);
  return Coord{s.x / n, s.y / n, s.z / n};
}

std::vector<int32_t> onetime_frames(const System& sys, int ts) {
  std::vector<int32_t> f;
  if (ts == -1) {
    for (int t = 0; t < sys.n_timesteps(); ++t) f.push_back(t);
  } else if (ts < -1) {
    f.push_back(-ts - 2);
  } else {
    for (int t = ts; t < sys.n_exponentials(); t += std::max(1, sys.n_exponential_steps())) f.push_back(t);
  }
  for (int t : f)
    if (t < 0 || t >= sys.n_timesteps()) throw Error(AMDAT_ERR_ARGUMENT, "time index out of range");
  return f;
}

}  // namespace amdat_host
