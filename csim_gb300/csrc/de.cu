// Differential evolution on the device (differentialEvolutionOptimizer.cpp:
// 216-468, deStrategy.cpp:23-158).
//
// State lives on the GPU: population [P][nvar] (candidate-major, i.e. the
// transpose of the reference's nvar x P matrix), objective values, trial
// population, the base ("original") population of the strategy, the best
// member, the population mean and spread, and a generation counter. A
// generation is csg_de_generate (permutations, mutation, binomial crossover,
// bounce-back) -> objective on the trial population -> csg_de_select (greedy
// selection, best member, statistics, counter + 1); all of it can be captured
// into one CUDA graph because every random number comes from a counter-based
// generator keyed by (seed, generation, stream, index) instead of host state.
//
// Random numbers: u = (splitmix64(key) >> 11) * 2^-53 in [0, 1). The
// reference draws from rand() and Armadillo's generator (not reproducible
// across platforms and racy inside OpenMP loops); the draws here are
// reproducible and the oracle restates the same generator, so trial vectors
// are compared bit for bit. Arithmetic uses explicit _rn intrinsics so no
// multiply-add is contracted.
#include <vector>

#include "ctx.hpp"

namespace csg {

enum DeStream : uint64_t { RS_SHUF1 = 1, RS_SHUF2 = 2, RS_COIN = 3, RS_CROSS = 4, RS_BOUNCE = 5,
                           RS_INIT = 6 };

__host__ __device__ inline uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__host__ __device__ inline double de_uniform(uint64_t seed, uint64_t gen, uint64_t stream,
                                             uint64_t idx) {
  uint64_t k = splitmix64(seed);
  k = splitmix64(k ^ gen);
  k = splitmix64(k ^ (stream << 56) ^ idx);
  return (double)(k >> 11) * (1.0 / 9007199254740992.0);
}

struct DeDev {
  int P, nvar;
  uint64_t seed;
  double* pop;
  double* f;
  double* trial;
  double* f_trial;
  double* orig;
  double* best;      // [nvar]
  double* best_val;  // [1]  (bestVal of the current stage)
  double* mean;      // [nvar]
  double* stats;     // [2]: mean and max distance from the mean
  double *glo, *ghi, *ilo, *ihi;  // [nvar] global and init bounds
  int* perm;         // [3][P] r1, r2, r3
  int* coin;         // [1]
  unsigned long long* gen;
  uint64_t draw = 0;  // extra trial sets of one generation (0: the standard draw)
};

// Shuffles (Fisher-Yates) and the either-or coin for one generation:
// deStrategy::makePopulationPermutations (deStrategy.cpp:23-65): slice 0 =
// pop[si1], slice i+1 = slice i's order rotated by si2(i) + 1.
__global__ void k_de_perm(DeDev d, int n_slices) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint64_t g = *d.gen ^ (d.draw << 48);
  const int P = d.P;
  int* si1 = d.perm;  // slice 0 order, built in place
  for (int i = 0; i < P; ++i) si1[i] = i;
  for (int i = P - 1; i > 0; --i) {
    const int j = (int)(de_uniform(d.seed, g, RS_SHUF1, i) * (double)(i + 1));
    const int t = si1[i];
    si1[i] = si1[j];
    si1[j] = t;
  }
  int si2[3] = {0, 1, 2};
  for (int i = n_slices - 1; i > 0; --i) {
    const int j = (int)(de_uniform(d.seed, g, RS_SHUF2, i) * (double)(i + 1));
    const int t = si2[i];
    si2[i] = si2[j];
    si2[j] = t;
  }
  // slice s index j -> si1[(j - shift_s) mod P], shift_s = sum_{i<s} (si2(i) + 1)
  int shift = 0;
  for (int s = 1; s < n_slices; ++s) {
    shift += si2[s - 1] + 1;
    for (int j = 0; j < P; ++j) d.perm[s * P + j] = si1[((j - shift) % P + P) % P];
  }
  *d.coin = de_uniform(d.seed, g, RS_COIN, 0) < 0.5 ? 1 : 0;
}

// Mutation (strategy), binomial crossover (:360-369) and bounce-back
// (:395-434) for every (candidate, variable).
__global__ void k_de_trial(DeDev d, int strategy, double fw, double cr) {
  const int P = d.P, nv = d.nvar;
  const uint64_t g = *d.gen ^ (d.draw << 48);
  const long long n = (long long)P * nv;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i / nv), v = (int)(i % nv);
    const double x = d.pop[i];
    double mut, orig;
    if (strategy == 1) {  // DE/local-to-best/1: x + F (best - x) + F (x_r1 - x_r2)
      const double a = d.pop[(long long)d.perm[c] * nv + v];
      const double b = d.pop[(long long)d.perm[P + c] * nv + v];
      const double t1 = __dmul_rn(fw, __dsub_rn(d.best[v], x));
      const double t2 = __dmul_rn(fw, __dsub_rn(a, b));
      mut = __dadd_rn(__dadd_rn(x, t1), t2);
      orig = x;
    } else {
      const double a = d.pop[(long long)d.perm[c] * nv + v];
      const double b = d.pop[(long long)d.perm[P + c] * nv + v];
      const double base = d.pop[(long long)d.perm[2 * P + c] * nv + v];
      if (strategy == 0 || *d.coin) {  // DE/rand/1: x_r3 + F (x_r1 - x_r2)
        mut = __dadd_rn(base, __dmul_rn(fw, __dsub_rn(a, b)));
      } else {  // either-or second branch: x_r3 + (F+1)/2 (x_r1 + x_r2 - 2 x_r3)
        const double k = __dmul_rn(0.5, __dadd_rn(fw, 1.0));
        mut = __dadd_rn(base, __dmul_rn(k, __dsub_rn(__dadd_rn(a, b), __dmul_rn(2.0, base))));
      }
      orig = base;
    }
    double cand = mut;
    if (cr < 1.0 && !(de_uniform(d.seed, g, RS_CROSS, i) < cr)) cand = x;
    // bounds: [mean + init bounds] clipped to the global bounds
    double up = __dadd_rn(d.mean[v], d.ihi[v]);
    double lo = __dadd_rn(d.mean[v], d.ilo[v]);
    if (up > d.ghi[v]) up = d.ghi[v];
    if (lo < d.glo[v]) lo = d.glo[v];
    if (cand < lo) {
      const double r = de_uniform(d.seed, g, RS_BOUNCE, i);
      cand = __dadd_rn(lo, __dmul_rn(r, __dsub_rn(orig, lo)));
    } else if (cand > up) {
      const double r = de_uniform(d.seed, g, RS_BOUNCE, i);
      cand = __dadd_rn(up, __dmul_rn(r, __dsub_rn(orig, up)));
    }
    d.trial[i] = cand;
    d.orig[i] = orig;
  }
}

// Greedy selection (:436-453), then (one block) the best member (:371-393),
// the population mean and distance statistics (compute_population_statistics)
// and the generation counter. initial != 0: no selection (fresh population).
__global__ void k_de_select(DeDev d, int initial) {
  const int P = d.P, nv = d.nvar;
  __shared__ int better[1024];
  for (int c = threadIdx.x; c < P; c += blockDim.x) {
    const bool b = !initial && d.f_trial[c] < d.f[c];
    better[c] = b;
    if (b) d.f[c] = d.f_trial[c];
  }
  __syncthreads();
  for (long long i = threadIdx.x; i < (long long)P * nv; i += blockDim.x) {
    const int c = (int)(i / nv);
    if (better[c]) d.pop[i] = d.trial[i];
  }
  __syncthreads();
  // best (lowest index among equal minima, as index_min)
  __shared__ double bv;
  __shared__ int bi;
  if (threadIdx.x == 0) {
    bv = d.f[0];
    bi = 0;
    for (int c = 1; c < P; ++c)
      if (d.f[c] < bv) {
        bv = d.f[c];
        bi = c;
      }
  }
  __syncthreads();
  const bool improve = bv < *d.best_val;
  for (int v = threadIdx.x; v < nv; v += blockDim.x) {
    if (improve) d.best[v] = d.pop[(long long)bi * nv + v];
    double s = 0.0;
    for (int c = 0; c < P; ++c) s += d.pop[(long long)c * nv + v];
    d.mean[v] = s / (double)P;
  }
  __syncthreads();
  if (threadIdx.x == 0 && improve) *d.best_val = bv;
  __shared__ double dist[1024];
  for (int c = threadIdx.x; c < P; c += blockDim.x) {
    double s = 0.0;
    for (int v = 0; v < nv; ++v) {
      const double e = d.pop[(long long)c * nv + v] - d.mean[v];
      s += e * e;
    }
    dist[c] = sqrt(s);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0, mx = 0.0;
    for (int c = 0; c < P; ++c) {
      m += dist[c];
      mx = fmax(mx, dist[c]);
    }
    d.stats[0] = m / (double)P;
    d.stats[1] = mx;
    if (!initial) *d.gen += 1;
  }
}

// init_population (:336-358): origin + spread (u - 0.5) (initUB - initLB)
// (uniform) or origin + spread n (initUB - initLB) (normal, Box-Muller).
__global__ void k_de_init(DeDev d, const double* origin, double spread, int type) {
  const int nv = d.nvar;
  const uint64_t g = *d.gen;
  const long long n = (long long)d.P * nv;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(i % nv);
    const double w = d.ihi[v] - d.ilo[v];
    double r;
    if (type == 0) {
      r = de_uniform(d.seed, g, RS_INIT, i) - 0.5;
    } else {
      const double u1 = 1.0 - de_uniform(d.seed, g, RS_INIT, 2 * i);
      const double u2 = de_uniform(d.seed, g, RS_INIT, 2 * i + 1);
      r = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
    d.pop[i] = __dadd_rn(origin[v], __dmul_rn(__dmul_rn(spread, r), w));
  }
}

}  // namespace csg

using namespace csg;

struct csg_de {
  csg_ctx* ctx = nullptr;
  DeDev d{};
  bool own_trial = true;
  std::vector<void*> allocs;
};

extern "C" {

int csg_de_create(csg_ctx* ctx, csg_de** out, int pop, int nvar, uint64_t seed) {
  CSG_CHECK(ctx && out, CSG_E_ARG, "csg_de_create: null argument");
  CSG_CHECK(pop >= 4 && pop <= 1024 && nvar > 0, CSG_E_SHAPE,
            "csg_de_create: population must be in [4, 1024]");
  DeviceGuard g(ctx->device);
  csg_de* de = new csg_de();
  de->ctx = ctx;
  DeDev& d = de->d;
  d.P = pop;
  d.nvar = nvar;
  d.seed = seed;
  const size_t pv = (size_t)pop * nvar;
  auto get = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    cudaMemsetAsync(p, 0, bytes, ctx->stream);
    de->allocs.push_back(p);
    return p;
  };
  d.pop = (double*)get(pv * 8);
  d.trial = (double*)get(pv * 8);
  d.orig = (double*)get(pv * 8);
  d.f = (double*)get(pop * 8);
  d.f_trial = (double*)get(pop * 8);
  d.best = (double*)get(nvar * 8);
  d.best_val = (double*)get(8);
  d.mean = (double*)get(nvar * 8);
  d.stats = (double*)get(16);
  d.glo = (double*)get(nvar * 8);
  d.ghi = (double*)get(nvar * 8);
  d.ilo = (double*)get(nvar * 8);
  d.ihi = (double*)get(nvar * 8);
  d.perm = (int*)get((size_t)3 * pop * 4);
  d.coin = (int*)get(4);
  d.gen = (unsigned long long*)get(8);
  for (void* p : de->allocs)
    if (!p) {
      for (void* q : de->allocs) cudaFree(q);
      delete de;
      set_error("csg_de_create: allocation failed");
      return CSG_E_NOMEM;
    }
  const double big = 1e300;
  CSG_CUDA(cudaMemcpyAsync(d.best_val, &big, 8, cudaMemcpyHostToDevice, ctx->stream));
  CSG_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = de;
  return CSG_OK;
}

int csg_de_destroy(csg_de* de) {
  if (!de) return CSG_OK;
  DeviceGuard g(de->ctx->device);
  cudaStreamSynchronize(de->ctx->stream);
  for (void* p : de->allocs) cudaFree(p);
  delete de;
  return CSG_OK;
}

int csg_de_set_bounds(csg_de* de, const double* global_lo, const double* global_hi,
                      const double* init_lo, const double* init_hi) {
  CSG_CHECK(de && global_lo && global_hi && init_lo && init_hi, CSG_E_ARG,
            "csg_de_set_bounds: null argument");
  CSG_CHECK(all_finite(global_lo, de->d.nvar) && all_finite(global_hi, de->d.nvar) &&
                all_finite(init_lo, de->d.nvar) && all_finite(init_hi, de->d.nvar),
            CSG_E_NAN, "csg_de_set_bounds: non-finite bound");
  DeviceGuard g(de->ctx->device);
  const size_t b = (size_t)de->d.nvar * 8;
  cudaStream_t st = de->ctx->stream;
  CSG_CUDA(cudaMemcpyAsync(de->d.glo, global_lo, b, cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(de->d.ghi, global_hi, b, cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(de->d.ilo, init_lo, b, cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(de->d.ihi, init_hi, b, cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaStreamSynchronize(st));
  return CSG_OK;
}

// Trial vectors are written to `trial` (device [P][nvar]) instead of the
// state's own buffer, e.g. straight into a chain's candidate-sag buffer.
int csg_de_set_trial_buffer(csg_de* de, double* trial) {
  CSG_CHECK(de && trial, CSG_E_ARG, "csg_de_set_trial_buffer: null argument");
  de->d.trial = trial;
  return CSG_OK;
}

int csg_de_buffers(csg_de* de, double** pop, double** f, double** trial, double** f_trial) {
  CSG_CHECK(de, CSG_E_ARG, "csg_de_buffers: null state");
  if (pop) *pop = de->d.pop;
  if (f) *f = de->d.f;
  if (trial) *trial = de->d.trial;
  if (f_trial) *f_trial = de->d.f_trial;
  return CSG_OK;
}

int csg_de_init(csg_de* de, const double* origin_host, double spread, int type) {
  CSG_CHECK(de && origin_host, CSG_E_ARG, "csg_de_init: null argument");
  CSG_CHECK(type == 0 || type == 1, CSG_E_ARG, "csg_de_init: type 0 (uniform) or 1 (normal)");
  DeviceGuard g(de->ctx->device);
  cudaStream_t st = de->ctx->stream;
  CSG_CUDA(cudaMemcpyAsync(de->d.mean, origin_host, (size_t)de->d.nvar * 8,
                           cudaMemcpyHostToDevice, st));
  const double big = 1e300;
  CSG_CUDA(cudaMemcpyAsync(de->d.best_val, &big, 8, cudaMemcpyHostToDevice, st));
  k_de_init<<<grid_for((long long)de->d.P * de->d.nvar, 256), 256, 0, st>>>(de->d, de->d.mean,
                                                                            spread, type);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int csg_de_generate_draw(csg_de* de, int strategy, double f_weight, double cr, int draw) {
  CSG_CHECK(de, CSG_E_ARG, "csg_de_generate: null state");
  CSG_CHECK(strategy >= 0 && strategy <= 2, CSG_E_ARG,
            "csg_de_generate: strategy 0 (rand/1), 1 (local-to-best/1) or 2 (either-or)");
  CSG_CHECK(draw >= 0 && draw < 65536, CSG_E_ARG, "csg_de_generate: draw out of range");
  DeviceGuard g(de->ctx->device);
  cudaStream_t st = de->ctx->stream;
  DeDev d = de->d;
  d.draw = (uint64_t)draw;
  k_de_perm<<<1, 32, 0, st>>>(d, strategy == 1 ? 2 : 3);
  CSG_LAUNCH_CHECK();
  k_de_trial<<<grid_for((long long)d.P * d.nvar, 256), 256, 0, st>>>(d, strategy, f_weight, cr);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int csg_de_generate(csg_de* de, int strategy, double f_weight, double cr) {
  return csg_de_generate_draw(de, strategy, f_weight, cr, 0);
}

int csg_de_select(csg_de* de, int initial) {
  CSG_CHECK(de, CSG_E_ARG, "csg_de_select: null state");
  DeviceGuard g(de->ctx->device);
  k_de_select<<<1, 256, 0, de->ctx->stream>>>(de->d, initial);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// Restart the current stage's best value (the reference sets bestVal = 1e15
// on a re-initialisation, differentialEvolutionOptimizer.cpp:251).
int csg_de_reset_best(csg_de* de) {
  CSG_CHECK(de, CSG_E_ARG, "csg_de_reset_best: null state");
  DeviceGuard g(de->ctx->device);
  const double big = 1e300;
  CSG_CUDA(cudaMemcpyAsync(de->d.best_val, &big, 8, cudaMemcpyHostToDevice, de->ctx->stream));
  return CSG_OK;
}

// Synchronous read of the state: best value, mean / max distance from the
// population mean, generation, and optionally the best vector (host nvar).
int csg_de_stats(csg_de* de, double* best_val, double* mean_dist, double* max_dist,
                 unsigned long long* generation, double* best_vec) {
  CSG_CHECK(de, CSG_E_ARG, "csg_de_stats: null state");
  DeviceGuard g(de->ctx->device);
  cudaStream_t st = de->ctx->stream;
  double bv = 0, s[2] = {0, 0};
  unsigned long long gen = 0;
  CSG_CUDA(cudaMemcpyAsync(&bv, de->d.best_val, 8, cudaMemcpyDeviceToHost, st));
  CSG_CUDA(cudaMemcpyAsync(s, de->d.stats, 16, cudaMemcpyDeviceToHost, st));
  CSG_CUDA(cudaMemcpyAsync(&gen, de->d.gen, 8, cudaMemcpyDeviceToHost, st));
  if (best_vec)
    CSG_CUDA(cudaMemcpyAsync(best_vec, de->d.best, (size_t)de->d.nvar * 8,
                             cudaMemcpyDeviceToHost, st));
  CSG_CUDA(cudaStreamSynchronize(st));
  if (best_val) *best_val = bv;
  if (mean_dist) *mean_dist = s[0];
  if (max_dist) *max_dist = s[1];
  if (generation) *generation = gen;
  return CSG_OK;
}

}  // extern "C"
