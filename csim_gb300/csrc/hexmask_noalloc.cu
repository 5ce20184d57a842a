// Hex focal-plane mask without any device allocation.
//
// csg_hex_mask allocates its per-call phasor buffer (one complex value per
// output and hex) with cudaMallocAsync. Some callers cannot let the library
// allocate: applications that reserve their whole device-memory budget at
// start-up so nothing can fail or stall for memory later (a wavefront-control
// loop running against a testbed, for instance), or host frameworks that hand
// the library only buffers they manage themselves. For them,
// csg_hex_mask_noalloc computes the same masks with the phasor scratch held in
// a fixed array in this file, which every GPU that loads the library keeps
// until the process exits.
#include <mutex>

#include "ctx.hpp"

namespace csg {
int hex_mask_with_phasor_buffer(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count, int S,
                                int n_sub, const double* sags, int n_hex, int n_out,
                                const int* cand, const double* lambda, double phase_sign, int flip,
                                double subtract, int use_only_hex, float* out, float2* phasors);
}  // namespace csg

using namespace csg;

// n_out * (n_hex + 1) phasors at most: 2 MiB of device memory per GPU.
static __device__ __align__(256) float2 g_hex_phasor_scratch[CSG_HEX_NOALLOC_MAX_PHASORS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
float2* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device`, looked up once per device
// with that device current (in host code the array's name is only a
// host-side stand-in, not a device address).
int scratch_for(int device, float2** out) {
  CSG_CHECK(device >= 0 && device < kMaxDevices, CSG_E_ARG,
            "csg_hex_mask_noalloc: device index out of range");
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[device]) {
    DeviceGuard g(device);
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_hex_phasor_scratch);
    CSG_CHECK(e == cudaSuccess && p != nullptr, CSG_E_CUDA,
              std::string("csg_hex_mask_noalloc: cudaGetSymbolAddress failed: ") +
                  cudaGetErrorString(e));
    g_scratch_ptr[device] = static_cast<float2*>(p);
  }
  *out = g_scratch_ptr[device];
  return CSG_OK;
}
}  // namespace

extern "C" int csg_hex_mask_noalloc(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count,
                                    int S, int n_sub, const double* sags, int n_hex, int n_out,
                                    const int* cand, const double* lambda, double phase_sign,
                                    int flip, double subtract, int use_only_hex, float* out) {
  CSG_CHECK(ctx && hex_id && count && sags && cand && lambda && out, CSG_E_ARG,
            "csg_hex_mask_noalloc: null argument");
  CSG_CHECK(S > 0 && n_sub > 0 && n_hex > 0 && n_hex < 32767 && n_out > 0, CSG_E_SHAPE,
            "csg_hex_mask_noalloc: bad shape");
  CSG_CHECK(use_only_hex >= -1 && use_only_hex <= n_hex, CSG_E_ARG,
            "csg_hex_mask_noalloc: use_only_hex out of range");
  CSG_CHECK((long long)n_out * (n_hex + 1) <= CSG_HEX_NOALLOC_MAX_PHASORS, CSG_E_SHAPE,
            "csg_hex_mask_noalloc: n_out * (n_hex + 1) = " +
                std::to_string((long long)n_out * (n_hex + 1)) + " exceeds the fixed scratch of " +
                std::to_string(CSG_HEX_NOALLOC_MAX_PHASORS) +
                " phasors; split the outputs over several calls or use csg_hex_mask");
  float2* scratch = nullptr;
  int rc = scratch_for(ctx->device, &scratch);
  if (rc) return rc;
  DeviceGuard g(ctx->device);
  // Every phasor the mask kernel reads is written earlier in the same call,
  // so the shared array needs no clearing between calls.
  return hex_mask_with_phasor_buffer(ctx, hex_id, count, S, n_sub, sags, n_hex, n_out, cand,
                                     lambda, phase_sign, flip, subtract, use_only_hex, out,
                                     scratch);
}
