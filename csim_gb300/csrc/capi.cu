// Context, memory, status and host<->device field transfer of the C ABI.
#include <cstring>
#include <string>

#include "ctx.hpp"

namespace csg {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
const char* get_error() { return g_last_error.c_str(); }

std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// Convert host complex<double> (interleaved, staged on device) to planar fp32.
// src: FP64 interleaved; colmajor: element (r, c, f) at r + c R + f R C.
__global__ void k_c128_to_c32p(const double2* __restrict__ src, float* __restrict__ dst, int R,
                               int C, int F, int colmajor) {
  const long long n = (long long)R * C * F;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    // i enumerates the destination in row-major [f][r][c]
    const int c = (int)(i % C);
    const long long t = i / C;
    const int r = (int)(t % R);
    const int f = (int)(t / R);
    const long long s = colmajor ? ((long long)f * R * C + (long long)c * R + r) : i;
    const double2 v = src[s];
    float* base = dst + (long long)f * 2 * R * C + (long long)r * C + c;
    base[0] = (float)v.x;
    base[(long long)R * C] = (float)v.y;
  }
}

__global__ void k_c32p_to_c128(const float* __restrict__ src, double2* __restrict__ dst, int R,
                               int C, int F, int colmajor) {
  const long long n = (long long)R * C * F;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long long t = i / C;
    const int r = (int)(t % R);
    const int f = (int)(t / R);
    const float* base = src + (long long)f * 2 * R * C + (long long)r * C + c;
    const long long d = colmajor ? ((long long)f * R * C + (long long)c * R + r) : i;
    dst[d] = make_double2((double)base[0], (double)base[(long long)R * C]);
  }
}

}  // namespace csg

using namespace csg;

extern "C" {

const char* csg_version(void) { return "csim_gb300 0.1 (sm_103a)"; }

unsigned long long csg_launch_count(void) { return g_launches.load(); }

int csg_profile(csg_ctx* c, int enable) {
  CSG_CHECK(c != nullptr, CSG_E_ARG, "csg_profile: null context");
  c->prof = enable != 0;
  if (enable) {
    c->acc.clear();
    for (auto& p : c->pending) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    c->pending.clear();
  }
  return CSG_OK;
}

int csg_profile_report(csg_ctx* c, char* buf, size_t len) {
  CSG_CHECK(c && buf && len > 0, CSG_E_ARG, "csg_profile_report: bad argument");
  DeviceGuard g(c->device);
  CSG_CUDA(cudaStreamSynchronize(c->stream));
  for (auto& p : c->pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, p.a, p.b);
    auto& a = c->acc[p.name];
    a.count += 1;
    a.ms += ms;
    a.flops += p.flops;
    a.bytes += p.bytes;
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  c->pending.clear();
  std::string s = "{";
  bool first = true;
  for (auto& kv : c->acc) {
    char tmp[256];
    snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"count\": %lld, \"ms\": %.6f, \"flops\": %.6e, \"bytes\": %.6e}",
             first ? "" : ", ", kv.first.c_str(), kv.second.count, kv.second.ms, kv.second.flops,
             kv.second.bytes);
    s += tmp;
    first = false;
  }
  s += "}";
  CSG_CHECK(s.size() + 1 <= len, CSG_E_ARG, "csg_profile_report: buffer too small");
  memcpy(buf, s.c_str(), s.size() + 1);
  return CSG_OK;
}

const char* csg_last_error(void) { return get_error(); }

int csg_create(csg_ctx** out, int device) {
  CSG_CHECK(out != nullptr, CSG_E_ARG, "csg_create: null output");
  int n = 0;
  CSG_CUDA(cudaGetDeviceCount(&n));
  CSG_CHECK(device >= 0 && device < n, CSG_E_ARG, "csg_create: bad device index");
  DeviceGuard g(device);
  csg_ctx* c = new csg_ctx();
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    return CSG_E_CUDA;
  }
  c->stream = c->own_stream;
  if (cudaMalloc(&c->status, sizeof(int)) != cudaSuccess ||
      cudaMemset(c->status, 0, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    cudaStreamDestroy(c->own_stream);
    delete c;
    set_error("csg_create: status word allocation failed");
    return CSG_E_NOMEM;
  }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return CSG_OK;
}

int csg_destroy(csg_ctx* c) {
  if (!c) return CSG_OK;
  DeviceGuard g(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  for (void* p : c->allocations) cudaFree(p);
  for (auto& kv : c->dft_plans) csg_mft_destroy(kv.second);
  if (c->dft_scratch) cudaFree(c->dft_scratch);
  if (c->dft_zero) cudaFree(c->dft_zero);
  for (int k = 0; k < 2; ++k) {
    if (c->ro_buf[k]) cudaFree(c->ro_buf[k]);
    if (c->ro_ready[k]) cudaEventDestroy(c->ro_ready[k]);
    if (c->ro_done[k]) cudaEventDestroy(c->ro_done[k]);
  }
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  cudaFree(c->status);
  cudaStreamDestroy(c->own_stream);
  delete c;
  return CSG_OK;
}

int csg_sync(csg_ctx* c) {
  CSG_CHECK(c != nullptr, CSG_E_ARG, "csg_sync: null context");
  DeviceGuard g(c->device);
  CSG_CUDA(cudaStreamSynchronize(c->stream));
  if (c->copy_stream) CSG_CUDA(cudaStreamSynchronize(c->copy_stream));
  int st = 0;
  CSG_CUDA(cudaMemcpy(&st, c->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (st != 0) {
    cudaMemset(c->status, 0, sizeof(int));
    set_error("device-side bounded wait ran out (code " + std::to_string(st) + ")");
    return CSG_E_TIMEOUT;
  }
  return CSG_OK;
}

int csg_set_wait_budget(csg_ctx* c, long long cycles) {
  CSG_CHECK(c != nullptr, CSG_E_ARG, "csg_set_wait_budget: null context");
  CSG_CHECK(cycles >= 0, CSG_E_ARG, "csg_set_wait_budget: cycles must be >= 0");
  c->wait_budget = cycles;
  return CSG_OK;
}

int csg_set_stream(csg_ctx* c, void* stream) {
  CSG_CHECK(c != nullptr, CSG_E_ARG, "csg_set_stream: null context");
  // NULL selects CUDA's default stream (stream 0), which is what torch's
  // default stream handle is; the context's own stream is used until this
  // call is made.
  c->stream = static_cast<cudaStream_t>(stream);
  return CSG_OK;
}

void* csg_get_stream(csg_ctx* c) { return c ? (void*)c->stream : nullptr; }

int csg_alloc(csg_ctx* c, size_t bytes, void** dptr) {
  CSG_CHECK(c && dptr, CSG_E_ARG, "csg_alloc: null argument");
  DeviceGuard g(c->device);
  void* p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
    cudaGetLastError();
    set_error("csg_alloc: cudaMalloc failed");
    return CSG_E_NOMEM;
  }
  c->allocations.insert(p);
  *dptr = p;
  return CSG_OK;
}

int csg_free(csg_ctx* c, void* p) {
  CSG_CHECK(c != nullptr, CSG_E_ARG, "csg_free: null context");
  if (!p) return CSG_OK;
  auto it = c->allocations.find(p);
  CSG_CHECK(it != c->allocations.end(), CSG_E_ARG, "csg_free: pointer not owned by context");
  DeviceGuard g(c->device);
  cudaStreamSynchronize(c->stream);
  c->allocations.erase(it);
  CSG_CUDA(cudaFree(p));
  return CSG_OK;
}

int csg_memcpy_h2d(csg_ctx* c, void* dst, const void* src, size_t bytes) {
  CSG_CHECK(c && dst && src, CSG_E_ARG, "csg_memcpy_h2d: null argument");
  DeviceGuard g(c->device);
  CSG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
  return CSG_OK;
}

int csg_memcpy_d2h(csg_ctx* c, void* dst, const void* src, size_t bytes) {
  CSG_CHECK(c && dst && src, CSG_E_ARG, "csg_memcpy_d2h: null argument");
  DeviceGuard g(c->device);
  CSG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
  return CSG_OK;
}

int csg_readout_d2h(csg_ctx* c, void* dst, const void* src, size_t bytes) {
  CSG_CHECK(c && dst && src, CSG_E_ARG, "csg_readout_d2h: null argument");
  DeviceGuard g(c->device);
  if (!bytes) return CSG_OK;
  if (!c->copy_stream) {
    CSG_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      CSG_CUDA(cudaEventCreateWithFlags(&c->ro_ready[k], cudaEventDisableTiming));
      CSG_CUDA(cudaEventCreateWithFlags(&c->ro_done[k], cudaEventDisableTiming));
    }
  }
  const int k = c->ro_next;
  c->ro_next ^= 1;
  if (c->ro_cap[k] < bytes) {
    // the buffer's last copy-out must finish before it is replaced
    CSG_CUDA(cudaEventSynchronize(c->ro_done[k]));
    if (c->ro_buf[k]) CSG_CUDA(cudaFree(c->ro_buf[k]));
    c->ro_buf[k] = nullptr;
    c->ro_cap[k] = 0;
    if (cudaMalloc(&c->ro_buf[k], bytes) != cudaSuccess) {
      cudaGetLastError();
      c->ro_buf[k] = nullptr;
      set_error("csg_readout_d2h: staging allocation failed");
      return CSG_E_NOMEM;
    }
    c->ro_cap[k] = bytes;
  }
  // staging k is free once its previous copy-out has run
  CSG_CUDA(cudaStreamWaitEvent(c->stream, c->ro_done[k], 0));
  CSG_CUDA(cudaMemcpyAsync(c->ro_buf[k], src, bytes, cudaMemcpyDeviceToDevice, c->stream));
  CSG_CUDA(cudaEventRecord(c->ro_ready[k], c->stream));
  CSG_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ro_ready[k], 0));
  CSG_CUDA(cudaMemcpyAsync(dst, c->ro_buf[k], bytes, cudaMemcpyDeviceToHost, c->copy_stream));
  CSG_CUDA(cudaEventRecord(c->ro_done[k], c->copy_stream));
  return CSG_OK;
}

int csg_memset(csg_ctx* c, void* dst, int value, size_t bytes) {
  CSG_CHECK(c && dst, CSG_E_ARG, "csg_memset: null argument");
  DeviceGuard g(c->device);
  CSG_CUDA(cudaMemsetAsync(dst, value, bytes, c->stream));
  return CSG_OK;
}

int csg_field_upload(csg_ctx* c, const double* host, int layout, int rows, int cols, int n_fields,
                     void* staging, float* dev_field) {
  CSG_CHECK(c && host && staging && dev_field, CSG_E_ARG, "csg_field_upload: null argument");
  CSG_CHECK(rows > 0 && cols > 0 && n_fields > 0, CSG_E_SHAPE, "csg_field_upload: bad shape");
  CSG_CHECK(layout == CSG_LAYOUT_COLMAJOR || layout == CSG_LAYOUT_ROWMAJOR, CSG_E_ARG,
            "csg_field_upload: bad layout");
  DeviceGuard g(c->device);
  const size_t n = (size_t)rows * cols * n_fields;
  CSG_CUDA(cudaMemcpyAsync(staging, host, n * 16, cudaMemcpyHostToDevice, c->stream));
  k_c128_to_c32p<<<grid_for(n, 256), 256, 0, c->stream>>>(
      static_cast<const double2*>(staging), dev_field, rows, cols, n_fields,
      layout == CSG_LAYOUT_COLMAJOR);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int csg_field_download(csg_ctx* c, const float* dev_field, int rows, int cols, int n_fields,
                       void* staging, double* host, int layout) {
  CSG_CHECK(c && host && staging && dev_field, CSG_E_ARG, "csg_field_download: null argument");
  CSG_CHECK(rows > 0 && cols > 0 && n_fields > 0, CSG_E_SHAPE, "csg_field_download: bad shape");
  CSG_CHECK(layout == CSG_LAYOUT_COLMAJOR || layout == CSG_LAYOUT_ROWMAJOR, CSG_E_ARG,
            "csg_field_download: bad layout");
  DeviceGuard g(c->device);
  const size_t n = (size_t)rows * cols * n_fields;
  k_c32p_to_c128<<<grid_for(n, 256), 256, 0, c->stream>>>(
      dev_field, static_cast<double2*>(staging), rows, cols, n_fields,
      layout == CSG_LAYOUT_COLMAJOR);
  CSG_LAUNCH_CHECK();
  CSG_CUDA(cudaMemcpyAsync(host, staging, n * 16, cudaMemcpyDeviceToHost, c->stream));
  return CSG_OK;
}

}  // extern "C"
