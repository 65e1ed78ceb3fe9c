// libtorch autograd functions over the engine's differentiable-structure entry
// points: a Gaussian-smoothed pair histogram and the auto structure factor of
// the |k| <= kmax lattice, each with a hand-written adjoint (gradient with
// respect to positions).  The forward and backward passes call the C ABI
// (amdat_gsmooth_run / amdat_gsmooth_adjoint, amdat_wave_density_lattice +
// amdat_structure_factor_run / amdat_structure_factor_adjoint) on the current
// CUDA stream; nothing here computes on the CPU.
//
// Positions: float32 CUDA tensor [frames][atoms][3], box [3] (float list), box
// origin 0.  Both functions reduce over all frames.  The smoothed histogram's
// pair loop is recomputed in the backward pass; the structure factor keeps its
// rho_k(t) table on the device until the backward pass has used it (or the
// graph is freed).
#include <ATen/cuda/CUDAContext.h>
#include <c10/cuda/CUDAGuard.h>
#include <torch/extension.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "amdat_gb300.h"

namespace {

void check(amdat_status st, const char* what) {
  TORCH_CHECK(st == AMDAT_OK, what, ": ", amdat_last_error());
}

// one engine context per device, on the caller's current stream
amdat_ctx* engine(int device) {
  static std::mutex mu;
  static std::map<int, amdat_ctx*> ctxs;
  std::lock_guard<std::mutex> lock(mu);
  auto it = ctxs.find(device);
  if (it == ctxs.end()) {
    amdat_ctx* c = nullptr;
    check(amdat_create(device, &c), "amdat_create");
    it = ctxs.emplace(device, c).first;
  }
  check(amdat_set_stream(it->second, at::cuda::getCurrentCUDAStream(device).stream()), "amdat_set_stream");
  return it->second;
}

void check_positions(const torch::Tensor& pos) {
  TORCH_CHECK(pos.is_cuda(), "positions must be a CUDA tensor");
  TORCH_CHECK(pos.scalar_type() == torch::kFloat32, "positions must be float32");
  TORCH_CHECK(pos.dim() == 3 && pos.size(2) == 3, "positions must be [frames][atoms][3]");
  TORCH_CHECK(pos.size(0) >= 1 && pos.size(1) >= 1, "need >= 1 frame and >= 1 atom");
}

// upload the positions as the context's trajectory; returns frames 0..F-1
std::vector<int32_t> upload(amdat_ctx* c, const torch::Tensor& pos, const std::vector<double>& box) {
  TORCH_CHECK(box.size() == 3, "box must have 3 entries");
  const float b[3] = {(float)box[0], (float)box[1], (float)box[2]};
  const float lo[3] = {0.f, 0.f, 0.f};
  check(amdat_traj_upload_device(c, (int32_t)pos.size(0), (int32_t)pos.size(1), pos.data_ptr<float>(), b, lo),
        "amdat_traj_upload_device");
  std::vector<int32_t> frames(pos.size(0));
  for (size_t f = 0; f < frames.size(); ++f) frames[f] = (int32_t)f;
  return frames;
}

class GSmooth : public torch::autograd::Function<GSmooth> {
 public:
  static torch::Tensor forward(torch::autograd::AutogradContext* actx, torch::Tensor pos,
                               std::vector<double> box, double sigma, double r_max, int64_t n_bins) {
    check_positions(pos);
    pos = pos.contiguous();
    const c10::cuda::CUDAGuard guard(pos.device());
    amdat_ctx* c = engine(pos.get_device());
    const auto frames = upload(c, pos, box);
    auto h = torch::empty({n_bins}, pos.options().dtype(torch::kFloat64));
    check(amdat_gsmooth_run(c, 0, frames.data(), (int32_t)frames.size(), (float)sigma, (float)r_max,
                            (int32_t)n_bins, AMDAT_OUT_DEVICE, h.data_ptr<double>()),
          "amdat_gsmooth_run");
    actx->save_for_backward({pos});
    actx->saved_data["box"] = box;
    actx->saved_data["sigma"] = sigma;
    actx->saved_data["r_max"] = r_max;
    actx->saved_data["n_bins"] = n_bins;
    return h;
  }

  static torch::autograd::tensor_list backward(torch::autograd::AutogradContext* actx,
                                               torch::autograd::tensor_list grads) {
    const torch::Tensor pos = actx->get_saved_variables()[0];
    const auto box = actx->saved_data["box"].toDoubleVector();
    const double sigma = actx->saved_data["sigma"].toDouble();
    const double r_max = actx->saved_data["r_max"].toDouble();
    const int64_t n_bins = actx->saved_data["n_bins"].toInt();
    const c10::cuda::CUDAGuard guard(pos.device());
    amdat_ctx* c = engine(pos.get_device());
    const auto frames = upload(c, pos, box);  // the pair loop is recomputed from the positions
    const torch::Tensor w = grads[0].to(torch::kFloat64).contiguous();
    auto g = torch::empty_like(pos);
    check(amdat_gsmooth_adjoint(c, 0, frames.data(), (int32_t)frames.size(), (float)sigma, (float)r_max,
                                (int32_t)n_bins, w.data_ptr<double>(), AMDAT_OUT_DEVICE, g.data_ptr<float>()),
          "amdat_gsmooth_adjoint");
    return {g, torch::Tensor(), torch::Tensor(), torch::Tensor(), torch::Tensor()};
  }
};

// keeps a density's rho table alive between the passes
struct DensityHold : torch::CustomClassHolder {
  amdat_ctx* ctx;
  int32_t handle;
  std::vector<int32_t> shell_off;
  DensityHold(amdat_ctx* c, int32_t h, std::vector<int32_t> off) : ctx(c), handle(h), shell_off(std::move(off)) {}
  ~DensityHold() override { amdat_wave_density_free(ctx, handle); }
};

class StructureFactor : public torch::autograd::Function<StructureFactor> {
 public:
  static torch::Tensor forward(torch::autograd::AutogradContext* actx, torch::Tensor pos,
                               std::vector<double> box, double kmax, double dk) {
    check_positions(pos);
    TORCH_CHECK(box.size() == 3 && box[0] == box[1] && box[1] == box[2], "structure factor needs a cubic box");
    pos = pos.contiguous();
    const c10::cuda::CUDAGuard guard(pos.device());
    amdat_ctx* c = engine(pos.get_device());
    const auto frames = upload(c, pos, box);
    int32_t h = 0, n_k = 0, n_shells = 0;
    check(amdat_wave_density_lattice(c, 0, (float)kmax, (float)dk, (float)box[0], frames.data(),
                                     (int32_t)frames.size(), AMDAT_MIXED, &h, &n_k, &n_shells),
          "amdat_wave_density_lattice");
    std::vector<int32_t> off(n_shells + 1);
    auto hold = c10::make_intrusive<DensityHold>(c, h, std::vector<int32_t>());
    check(amdat_wave_density_vectors(c, h, nullptr, off.data()), "amdat_wave_density_vectors");
    hold->shell_off = off;
    auto s = torch::empty({n_shells}, pos.options().dtype(torch::kFloat64));
    check(amdat_structure_factor_run(c, h, h, off.data(), n_shells, AMDAT_OUT_DEVICE, s.data_ptr<double>()),
          "amdat_structure_factor_run");
    actx->saved_data["density"] = c10::IValue::make_capsule(hold);
    actx->saved_data["box"] = box;
    actx->save_for_backward({pos});
    return s;
  }

  static torch::autograd::tensor_list backward(torch::autograd::AutogradContext* actx,
                                               torch::autograd::tensor_list grads) {
    auto hold = c10::static_intrusive_pointer_cast<DensityHold>(actx->saved_data["density"].toCapsule());
    const torch::Tensor pos = actx->get_saved_variables()[0];
    const auto box = actx->saved_data["box"].toDoubleVector();
    const c10::cuda::CUDAGuard guard(pos.device());
    amdat_ctx* c = engine(pos.get_device());
    upload(c, pos, box);  // the phases are taken from the saved positions
    const torch::Tensor w = grads[0].to(torch::kFloat64).contiguous();
    auto g = torch::empty_like(pos);
    check(amdat_structure_factor_adjoint(c, hold->handle, hold->shell_off.data(),
                                         (int32_t)hold->shell_off.size() - 1, w.data_ptr<double>(),
                                         AMDAT_OUT_DEVICE, g.data_ptr<float>()),
          "amdat_structure_factor_adjoint");
    return {g, torch::Tensor(), torch::Tensor(), torch::Tensor()};
  }
};

torch::Tensor gsmooth(torch::Tensor pos, std::vector<double> box, double sigma, double r_max, int64_t n_bins) {
  return GSmooth::apply(pos, box, sigma, r_max, n_bins);
}

torch::Tensor structure_factor(torch::Tensor pos, std::vector<double> box, double kmax, double dk) {
  return StructureFactor::apply(pos, box, kmax, dk);
}

// shell offsets and vectors of the lattice the structure factor uses
std::vector<torch::Tensor> lattice(torch::Tensor pos, std::vector<double> box, double kmax, double dk) {
  check_positions(pos);
  pos = pos.contiguous();
  const c10::cuda::CUDAGuard guard(pos.device());
  amdat_ctx* c = engine(pos.get_device());
  const auto frames = upload(c, pos.narrow(0, 0, 1).contiguous(), box);
  int32_t h = 0, n_k = 0, n_shells = 0;
  check(amdat_wave_density_lattice(c, 0, (float)kmax, (float)dk, (float)box[0], frames.data(), 1, AMDAT_MIXED,
                                   &h, &n_k, &n_shells),
        "amdat_wave_density_lattice");
  auto kv = torch::empty({n_k, 3}, torch::kInt32);
  auto off = torch::empty({n_shells + 1}, torch::kInt32);
  const amdat_status st = amdat_wave_density_vectors(c, h, kv.data_ptr<int32_t>(), off.data_ptr<int32_t>());
  amdat_wave_density_free(c, h);
  check(st, "amdat_wave_density_vectors");
  return {kv, off};
}

// per-kernel device timing and launch count of the device's engine context
void profile_reset(bool enable, int64_t device) {
  check(amdat_profile_reset(engine((int)device), enable ? 1 : 0), "amdat_profile_reset");
}

std::pair<int64_t, double> profile_kernel(const std::string& name, int64_t device) {
  int64_t n = 0;
  double ms = 0.0;
  check(amdat_profile_kernel(engine((int)device), name.c_str(), &n, &ms), "amdat_profile_kernel");
  return {n, ms};
}

int64_t launch_count(int64_t device) {
  int64_t n = 0;
  check(amdat_launch_count(engine((int)device), &n), "amdat_launch_count");
  return n;
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
  m.doc() = "autograd functions over the amdat_gb300 differentiable-structure kernels";
  m.def("gsmooth", &gsmooth, "Gaussian-smoothed pair histogram h[n_bins] (float64), differentiable",
        py::arg("pos"), py::arg("box"), py::arg("sigma"), py::arg("r_max"), py::arg("n_bins"));
  m.def("structure_factor", &structure_factor,
        "S_raw per shell (sum over frames and shell vectors of |rho_k|^2 / H_s), differentiable",
        py::arg("pos"), py::arg("box"), py::arg("kmax"), py::arg("dk"));
  m.def("lattice", &lattice, "lattice vectors [n_k][3] and shell offsets of the structure factor",
        py::arg("pos"), py::arg("box"), py::arg("kmax"), py::arg("dk"));
  m.def("profile_reset", &profile_reset, "enable/disable and clear per-kernel timing", py::arg("enable"),
        py::arg("device") = 0);
  m.def("profile_kernel", &profile_kernel, "(launches, total ms) of a kernel since the last reset",
        py::arg("name"), py::arg("device") = 0);
  m.def("launch_count", &launch_count, "kernels launched by the engine context", py::arg("device") = 0);
}
