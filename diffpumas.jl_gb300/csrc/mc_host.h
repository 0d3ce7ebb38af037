// mc_host.h -- host side shared by the backward MC translation units (mc.cu:
// two-layer geometry of run_backward_mc; dir_mc.cu: fixed directional paths):
// prepared media, their packed device layout, run checks and the
// per-group tallies.
#pragma once
#include <cstdint>
#include <vector>

#include "internal.h"
#include "mc_device.cuh"

// A prepared medium (one material or a runtime mixture, src/Types.jl:357-376,
// with its MIXED transport kernel, src/MixedTransport.jl:51-97): host columns
// plus device blobs cached per partner medium.
struct dp_mixture {
  const dp_physics* phys = nullptr;
  uint64_t uid = 0;
  int nm = 0;
  std::vector<int> mats;
  std::vector<double> fracs;
  int n = 0;                  // physics grid nodes
  std::vector<double> cols;   // (MC_LB1 + 2*nm) columns of n: see MedCol
  int nk = 0;                 // MIXED kernel nodes
  std::vector<double> kcols;  // K_NCOL columns of nk
  double onset = 0, ZoA = 0;
  std::vector<double> el;     // nel x kElStride
  int nel = 0;
  struct Blob {
    uint64_t partner, partner2;  // air medium, porous medium (0: none)
    int precision;
    unsigned char* dev;
    dp::mc::Layout lay;
  };
  std::vector<Blob> blobs;    // this medium as rock, `partner` as air, `partner2` as porous
};

namespace dp {
namespace mc {

// One packed layout for every medium of a launch (the widest mixture sets
// the transport-path slots); esize is sizeof the transport precision.
Layout make_layout(const dp_mixture* const* media, int n_media, size_t esize);
// Packs medium m into med_bytes at out.
void pack_medium(const dp_mixture* m, const Layout& L, size_t esize, unsigned char* out);
MedInfo make_info(const dp_mixture* m);
// Checks a run configuration and fills the run constants; thr_fp64 receives
// the FP64 source-energy ceiling.
int check_cfg(dp_ctx* ctx, const dp_physics* ph, const dp_mc_config* cfg, Consts* C,
              double* thr_fp64 = nullptr);
// Synchronises; DP_ERR_STATE if a kernel raised the context's error flag.
int read_flag(dp_ctx* ctx);
// The call's result for the OR of the histories' status bits.
int status_code(dp_ctx* ctx, int bits);
// read_flag, then status_code of the device word d_bits.
int status_result(dp_ctx* ctx, const int* d_bits);
// Per-group tallies (groups: lines of sight or directions).  group_offsets
// writes the running sample offsets (from the lines of sight's n_samples, or
// copied from `given`) and the tally-chunk offsets; group_tally reduces the
// per-history contributions of each group in a fixed order.
int group_offsets(dp_ctx* ctx, const dp_los* los, const int64_t* given, long n, int64_t* off,
                  int64_t* coff, long expect);
long tally_jobs(long n, long total);
size_t tally_part_bytes();
int group_tally(dp_ctx* ctx, const double* contrib, const int32_t* status, const double* csda,
                const double* dcsda, const dp_los* los, const int32_t* valid, long n, long total,
                int sigma_n1, const int64_t* off, const int64_t* coff, void* part,
                dp_los_result* out, int* bits);

}  // namespace mc
}  // namespace dp
