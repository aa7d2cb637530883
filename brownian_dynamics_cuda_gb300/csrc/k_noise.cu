// The reference's noise stream generated on the device.
//
// main.cpp:479-486 draws, per step, two uniforms on LH-Monte-Carlo steps
// (step % 100 == 0, main.cpp:387-388), then 3n rotational deviates
// (normal(0, r_var[i])) and 3 n_D translational ones (normal(0, 1)), from
// one MT19937 (Matsumoto & Nishimura 1998; mt.cpp:93-141) through the polar
// Box-Muller method with a cached second deviate (utilities.cpp:304-336).
// Here one CTA per generator keeps the 624-word state in shared memory:
//   twist      the state update in four barrier-separated phases (words
//              [0,227) read only old words; [227,454) and [454,623) read the
//              words 227 below them, rewritten by the previous phase; 623
//              last), each phase reading into registers before writing;
//   pairs      the tempered words of the block, plus a word carried over
//              from the previous block, form candidate (x, y) pairs, one
//              thread each; acceptance (0 < x^2 + y^2 <= 1) and a block scan
//              place the accepted pairs' two deviates in output order;
//              consumption stops at exactly the pair that completes the
//              step, whose second deviate becomes the cache.
// The 32-bit stream and the accept / reject decisions are the host's bit
// for bit.  The logarithm is the correctly rounded one of cr_log.cuh, so
// the deviates equal a host stream set to BD_LOG_CR bit for bit, and the
// reference's (the C library's log) wherever that log rounds correctly.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "bd_internal.h"
#include "cr_log.cuh"

using bdh::set_error;

#define CK(call)                                                                                 \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) {                                                                     \
      char b_[256];                                                                              \
      snprintf(b_, sizeof b_, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return set_error(e_ == cudaErrorMemoryAllocation ? BD_ERR_NOMEM : BD_ERR_CUDA, b_);        \
    }                                                                                            \
  } while (0)

namespace {

constexpr int kN = 624, kM = 397;
constexpr int kThreads = 320;  // >= 313 candidate pairs per block

struct DevMt {
  uint32_t st[kN];
  int idx;      // next word of the current block (kN: twist first)
  int have;     // a cached deviate is pending
  double cached;
};

__device__ __forceinline__ uint32_t mix(uint32_t a, uint32_t b, uint32_t c) {
  const uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
  return c ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

__device__ __forceinline__ uint32_t temper(uint32_t y) {
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

// in-place twist of st[] by the whole CTA
__device__ void twist(uint32_t* st) {
  const int t = threadIdx.x;
  uint32_t v[2];
  // words [0, 227): old words only
  for (int k = 0; k < 2; k++) {
    const int i = t + k * kThreads;
    if (i < kN - kM) v[k] = mix(st[i], st[i + 1], st[i + kM]);
  }
  __syncthreads();
  for (int k = 0; k < 2; k++) {
    const int i = t + k * kThreads;
    if (i < kN - kM) st[i] = v[k];
  }
  __syncthreads();
  // words [227, 454), then [454, 623): st[i + 1] old, st[i - 227] new
  for (int ph = 0; ph < 2; ph++) {
    const int lo = (kN - kM) * (ph + 1), hi = ph == 0 ? 2 * (kN - kM) : kN - 1;
    for (int k = 0; k < 2; k++) {
      const int i = lo + t + k * kThreads;
      if (i < hi) v[k] = mix(st[i], st[i + 1], st[i - (kN - kM)]);
    }
    __syncthreads();
    for (int k = 0; k < 2; k++) {
      const int i = lo + t + k * kThreads;
      if (i < hi) st[i] = v[k];
    }
    __syncthreads();
  }
  if (t == 0) st[kN - 1] = mix(st[kN - 1], st[0], st[kM - 1]);
  __syncthreads();
}

__device__ __forceinline__ void emit(int i, double z, int n3, const double* r_var, double* rr, double* p) {
  if (i < n3) rr[i] = __dadd_rn(__dmul_rn(z, r_var[i]), 0.0);
  else p[i - n3] = __dadd_rn(__dmul_rn(z, 1.0), 0.0);
}

__device__ __forceinline__ void mt_noise_body(DevMt* G, int step, int n3, const double* __restrict__ r_var, int nD3,
                                              double* rr, double* p) {
  __shared__ uint32_t st[kN];
  __shared__ int s_idx, s_have, s_o, s_carry_ok, s_stop;
  __shared__ uint32_t s_carry;
  __shared__ double s_cached;
  __shared__ int wsum[kThreads / 32];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  for (int i = t; i < kN; i += kThreads) st[i] = G->st[i];
  if (t == 0) {
    s_idx = G->idx;
    s_have = G->have;
    s_cached = G->cached;
    s_o = 0;
    s_carry_ok = 0;
  }
  __syncthreads();
  const int N = n3 + nD3;
  if (step % 100 == 0) {  // two uniforms for the LH Monte Carlo, discarded here
    int skip = 2;
    while (skip > 0) {
      if (s_idx >= kN) {
        twist(st);
        if (t == 0) s_idx = 0;
        __syncthreads();
      }
      const int take = min(skip, kN - s_idx);
      skip -= take;
      __syncthreads();
      if (t == 0) s_idx += take;
      __syncthreads();
    }
  }
  if (t == 0 && s_have && N > 0) {
    emit(0, s_cached, n3, r_var, rr, p);
    s_have = 0;
    s_o = 1;
  }
  __syncthreads();
  const double C = 1.0 / 4294967295.0;
  while (s_o < N) {
    if (s_idx >= kN) {
      twist(st);
      if (t == 0) s_idx = 0;
      __syncthreads();
    }
    const int idx = s_idx, cok = s_carry_ok, o = s_o;
    const int len = (kN - idx) + cok;
    const int P = len / 2;
    const int need = N - o, np = (need + 1) / 2;
    double x = 0.0, y = 0.0, q = 0.0;
    int acc = 0;
    if (t < P) {
      const int j0 = 2 * t, j1 = 2 * t + 1;
      const uint32_t a = (cok && j0 == 0) ? s_carry : temper(st[idx + j0 - cok]);
      const uint32_t b = temper(st[idx + j1 - cok]);
      x = __dadd_rn(__dmul_rn(2.0, __dmul_rn((double)a, C)), -1.0);
      y = __dadd_rn(__dmul_rn(2.0, __dmul_rn((double)b, C)), -1.0);
      q = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
      acc = !(q == 0.0 || q > 1.0);
    }
    // exclusive rank of this pair among the accepted ones
    const unsigned bal = __ballot_sync(0xffffffffu, acc);
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < kThreads / 32; w++) {
      if (w < wid) before += wsum[w];
      total += wsum[w];
    }
    const int r = before + __popc(bal & ((1u << lane) - 1u));
    if (total >= np) {
      // the pair of rank np - 1 completes the step
      if (acc && r == np - 1) s_stop = t;
      __syncthreads();
      const int kstop = s_stop;
      if (acc && r < np) {
        const double d = sqrt(-2.0 * crlog::log_cr(q) / q);
        const double zx = __dmul_rn(x, d), zy = __dmul_rn(y, d);
        const int i0 = o + 2 * r;
        emit(i0, zx, n3, r_var, rr, p);
        if (i0 + 1 < N) {
          emit(i0 + 1, zy, n3, r_var, rr, p);
        } else {
          s_cached = zy;
          s_have = 1;
        }
      }
      if (t == 0) {
        s_idx = idx + 2 * (kstop + 1) - cok;
        s_carry_ok = 0;
        s_o = N;
      }
    } else {
      if (acc) {
        const double d = sqrt(-2.0 * crlog::log_cr(q) / q);
        emit(o + 2 * r, __dmul_rn(x, d), n3, r_var, rr, p);
        emit(o + 2 * r + 1, __dmul_rn(y, d), n3, r_var, rr, p);
      }
      if (t == 0) {
        if (len & 1) {
          s_carry = temper(st[kN - 1]);
          s_carry_ok = 1;
        } else {
          s_carry_ok = 0;
        }
        s_idx = kN;
        s_o = o + 2 * total;
      }
    }
    __syncthreads();
  }
  for (int i = t; i < kN; i += kThreads) G->st[i] = st[i];
  if (t == 0) {
    G->idx = s_idx;
    G->have = s_have;
    G->cached = s_cached;
  }
}

__global__ void __launch_bounds__(kThreads) k_mt_noise(DevMt* G, int step, int n3, const double* __restrict__ r_var,
                                                        int nD3, double* rr, double* p) {
  mt_noise_body(G, step, n3, r_var, nD3, rr, p);
}

// one generator per CTA: every replica's step in one launch
struct NoiseJob {
  DevMt* G;
  const double* r_var;
  double* rr;
  double* p;
  int n3, nD3;
};

__global__ void __launch_bounds__(kThreads) k_mt_noise_multi(const NoiseJob* __restrict__ jobs, int step) {
  const NoiseJob j = jobs[blockIdx.x];
  mt_noise_body(j.G, step, j.n3, j.r_var, j.nD3, j.rr, j.p);
}

DevMt seeded(unsigned long seed) {
  bdh::Mt19937 h;
  h.seed((uint32_t)(seed & 0xffffffffUL));
  DevMt m;
  std::memcpy(m.st, h.st, sizeof m.st);
  m.idx = h.idx >= kN ? kN : h.idx;
  m.have = 0;
  m.cached = 0.0;
  return m;
}

}  // namespace

// Noise of a whole batch: generator i seeded seeds[i] writes n3[i] scaled
// rotational draws into d_rr[i] and nD3[i] translational ones into d_p[i]
// (the replica contexts' own noise buffers), all in one launch per step.
struct bdk::NoiseBatch {
  int nr = 0;
  DevMt* G = nullptr;
  NoiseJob* jobs = nullptr;
  double* rvar = nullptr;
};

int bdk::noise_batch_create(int nr, const unsigned long* seeds, const int* n3, const int* nD3,
                            const double* const* h_rvar, double* const* d_rr, double* const* d_p, NoiseBatch** out) {
  NoiseBatch* b = new NoiseBatch();
  b->nr = nr;
  size_t nv = 0;
  for (int i = 0; i < nr; i++) nv += (size_t)n3[i];
  std::vector<DevMt> g(nr);
  for (int i = 0; i < nr; i++) g[i] = seeded(seeds[i]);
  std::vector<NoiseJob> jobs(nr);
  std::vector<double> rv(nv);
  cudaError_t e = cudaMalloc(&b->G, nr * sizeof(DevMt));
  if (e == cudaSuccess) e = cudaMalloc(&b->jobs, nr * sizeof(NoiseJob));
  if (e == cudaSuccess && nv) e = cudaMalloc(&b->rvar, nv * sizeof(double));
  if (e != cudaSuccess) {
    noise_batch_free(b);
    return set_error(BD_ERR_NOMEM, "noise batch: cudaMalloc failed");
  }
  size_t o = 0;
  for (int i = 0; i < nr; i++) {
    std::memcpy(rv.data() + o, h_rvar[i], n3[i] * sizeof(double));
    jobs[i] = NoiseJob{b->G + i, b->rvar + o, d_rr[i], d_p[i], n3[i], nD3[i]};
    o += (size_t)n3[i];
  }
  e = cudaMemcpy(b->G, g.data(), nr * sizeof(DevMt), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->jobs, jobs.data(), nr * sizeof(NoiseJob), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && nv) e = cudaMemcpy(b->rvar, rv.data(), nv * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    noise_batch_free(b);
    return set_error(BD_ERR_CUDA, "noise batch: upload failed");
  }
  *out = b;
  return BD_OK;
}

int bdk::noise_batch_step(NoiseBatch* b, int step, cudaStream_t st) {
  if (!b || b->nr == 0) return BD_OK;
  k_mt_noise_multi<<<b->nr, kThreads, 0, st>>>(b->jobs, step);
  CK(cudaGetLastError());
  return BD_OK;
}

void bdk::noise_batch_free(NoiseBatch* b) {
  if (!b) return;
  if (b->G) cudaFree(b->G);
  if (b->jobs) cudaFree(b->jobs);
  if (b->rvar) cudaFree(b->rvar);
  delete b;
}

struct bd_dev_noise {
  DevMt* d = nullptr;
};

extern "C" int bd_dev_noise_create(unsigned long seed, bd_dev_noise** out) {
  if (!out) return set_error(BD_ERR_ARG, "bd_dev_noise_create: null argument");
  const DevMt m = seeded(seed);
  bd_dev_noise* g = new bd_dev_noise();
  cudaError_t e = cudaMalloc(&g->d, sizeof(DevMt));
  if (e != cudaSuccess) {
    delete g;
    return set_error(BD_ERR_NOMEM, "bd_dev_noise_create: cudaMalloc failed");
  }
  e = cudaMemcpy(g->d, &m, sizeof m, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(g->d);
    delete g;
    return set_error(BD_ERR_CUDA, "bd_dev_noise_create: upload failed");
  }
  *out = g;
  return BD_OK;
}

extern "C" int bd_dev_noise_step(bd_dev_noise* g, int step, int n3, const double* d_r_var, int n_D3, double* d_rr,
                                 double* d_p, void* stream) {
  if (!g || n3 < 0 || n_D3 < 0 || (n3 > 0 && (!d_r_var || !d_rr)) || (n_D3 > 0 && !d_p))
    return set_error(BD_ERR_ARG, "bd_dev_noise_step: bad argument");
  k_mt_noise<<<1, kThreads, 0, (cudaStream_t)stream>>>(g->d, step, n3, d_r_var, n_D3, d_rr, d_p);
  CK(cudaGetLastError());
  return BD_OK;
}

extern "C" int bd_dev_noise_free(bd_dev_noise* g) {
  if (!g) return BD_OK;
  if (g->d) cudaFree(g->d);
  delete g;
  return BD_OK;
}
