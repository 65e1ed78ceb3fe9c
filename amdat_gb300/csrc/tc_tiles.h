// Tiling of a half-space lattice for the tensor-core kernels (shared by the
// forward rho_k kernel and the S(k) adjoint): 8 x 8 (nx, ny) row blocks times
// nz windows, each tile trimmed to a multiple of 16 nz columns.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "engine.h"

namespace amdat {

struct TcTile {
  int32_t nx0, ny0, zblk, entry0;  // entry map: 64 rows x n ints from entry0 (vector index or -1)
  int32_t n, pad0, pad1, pad2;     // nz columns of this tile (multiple of 16, <= 128)
};

struct TcPlan {
  DevBuf<TcTile> tiles;
  DevBuf<int32_t> entry_k;
  std::vector<TcTile> host_tiles;
  int32_t n_tiles = 0, n_zblk = 0, nzw = 0, nmax = 0;
  int64_t entries = 0;  // rows x columns computed per frame and atom, padding included
};

TcPlan* tc_plan_build(const std::vector<int32_t>& kvec);
void tc_plan_free(TcPlan* p);
// the tensor-core tiling of a lattice density's plan (built at first use)
TcPlan* lattice_tc_plan(amdat_ctx* ctx, const std::string& lattice_key);
// whether the tensor-core kernels run (compute capability 10.x and not
// disabled through AMDAT_RHOK_KERNEL=fp32)
bool tc_enabled(amdat_ctx* ctx);

}  // namespace amdat
