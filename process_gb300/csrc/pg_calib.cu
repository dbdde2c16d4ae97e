// Expected-VAF binomial-mixture likelihood of an alt/depth table and its
// adjoint, batched over replicates (no reference counterpart: ProCESS has no
// calibration path; this is the differentiable form of the sequencing output
// used to fit epoch rates, exposures and purity to observed VAFs).
//
// Model of replicate r with K epochs, J signatures S_j over C classes:
//   w_k      = softmax(theta_k)                   (exposures of epoch k)
//   M_k(c)   = sum_j w_kj S_j(c)
//   pi_k(c)  = exp(lr_k) L_k M_k(c) / Z,   Z = sum_k exp(lr_k) L_k
//   v_k      = sigmoid(rho) phi_k / 2              (expected VAF of epoch k)
//   NLL      = - sum_i log sum_k pi_k(c_i) v_k^a_i (1 - v_k)^(d_i - a_i)
// (the binomial coefficient, constant in the parameters, is left out).
// Parameters per replicate, in order: lr_0..K-1, theta_00..theta_K-1,J-1, rho.
//
// Kernels: k_calib_sites (one CTA per (replicate, chunk of sites)) computes
// per-site log-likelihoods and responsibilities gamma_k in FP32 and reduces
//   G_k(c) = sum_{i: c_i = c} gamma_ik,  A_k = sum gamma_ik a_i,
//   B_k = sum gamma_ik (d_i - a_i),  NLL
// with per-thread Neumaier-compensated sums and deterministic per-warp class
// bins; k_calib_epilogue (one CTA per replicate) adds the chunk partials in a
// fixed order (compensated) and applies the chain rule, optionally followed
// by an Adam step on the parameters.
#include <cstdint>

#include "pg_kernels.h"

namespace pg {

constexpr int CAL_THREADS = 256;
constexpr int CAL_WARPS = CAL_THREADS / 32;
constexpr uint32_t CAL_MAXK = 8, CAL_MAXJ = 8, CAL_MAXC = 128;

struct Neu {   // Neumaier-compensated FP32 sum
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ float value() const { return s + c; }
};

// per-replicate derived tables: log pi_k(c), log v_k, log(1 - v_k)
__device__ void calib_tables(const CalibArgs& a, uint32_t r, const float* __restrict__ p, float* logpi, float* lv,
                             float* l1v) {
  const uint32_t K = a.K, J = a.J, C = a.C;
  // Z and softmax are tiny: every thread recomputes them
  float Z = 0.f;
  for (uint32_t k = 0; k < K; ++k) Z += expf(p[k]) * a.epoch_w[r * K + k];
  const float lZ = logf(Z);
  const float sig = 1.f / (1.f + expf(-p[K + K * J]));
  for (uint32_t x = threadIdx.x; x < K * C; x += blockDim.x) {
    const uint32_t k = x / C, c = x % C;
    const float* th = p + K + k * J;
    float mx = th[0];
    for (uint32_t j = 1; j < J; ++j) mx = fmaxf(mx, th[j]);
    float den = 0.f, num = 0.f;
    for (uint32_t j = 0; j < J; ++j) {
      const float e = expf(th[j] - mx);
      den += e;
      num += e * a.sig[j * C + c];
    }
    const float M = num / den;
    logpi[c * K + k] = p[k] + logf(a.epoch_w[r * K + k]) + logf(fmaxf(M, 1e-30f)) - lZ;   // class-major
  }
  if (threadIdx.x < K) {
    const float v = sig * a.phi[r * K + threadIdx.x] * 0.5f;
    lv[threadIdx.x] = logf(v);
    l1v[threadIdx.x] = log1pf(-v);
  }
}

// K floats as one vector access where K is a multiple of 4
template <uint32_t K, bool V = (K % 4 == 0)> struct KVec {
  using type = float;
  __device__ static void load(const float* p, float* v) {
#pragma unroll
    for (uint32_t k = 0; k < K; ++k) v[k] = p[k];
  }
  __device__ static void add(float* p, const float* v) {
#pragma unroll
    for (uint32_t k = 0; k < K; ++k) p[k] += v[k];
  }
};
template <uint32_t K> struct KVec<K, true> {
  using type = float4;
  __device__ static void load(const float* p, float* v) {
#pragma unroll
    for (uint32_t k = 0; k < K; k += 4) {
      const float4 x = *reinterpret_cast<const float4*>(p + k);
      v[k] = x.x; v[k + 1] = x.y; v[k + 2] = x.z; v[k + 3] = x.w;
    }
  }
  __device__ static void add(float* p, const float* v) {
#pragma unroll
    for (uint32_t k = 0; k < K; k += 4) {
      float4 x = *reinterpret_cast<float4*>(p + k);
      x.x += v[k]; x.y += v[k + 1]; x.z += v[k + 2]; x.w += v[k + 3];
      *reinterpret_cast<float4*>(p + k) = x;
    }
  }
};

// Per-site work: every thread takes sites i0 + tid, i0 + tid + 256, ...
// (coalesced), keeps plain FP32 sums over its ~32 sites, and adds its
// responsibilities straight into its warp's class bins; lanes of one warp
// that share a class add theirs in lane order (deterministic).  The sums are
// compensated from the warp level on.
template <uint32_t K>
__global__ void __launch_bounds__(CAL_THREADS) k_calib_sites(CalibArgs a, const float* __restrict__ params,
                                                             const uint32_t* __restrict__ chunk_rep,
                                                             const uint64_t* __restrict__ chunk_start,
                                                             float* __restrict__ partial) {
  __shared__ __align__(16) float s_logpi[K * CAL_MAXC];
  __shared__ float s_lv[K], s_l1v[K];
  __shared__ __align__(16) float s_bins[CAL_WARPS][K * CAL_MAXC];
  __shared__ float s_red[CAL_WARPS][2 + 4 * K];
  const uint32_t chunk = a.chunk0 + blockIdx.x;
  const uint32_t r = chunk_rep[chunk];
  const uint64_t i0 = chunk_start[chunk];
  const uint64_t i1 = min(i0 + a.chunk, a.site_off[r + 1]);
  const uint32_t C = a.C, P = a.P;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  calib_tables(a, r, params + uint64_t(r) * P, s_logpi, s_lv, s_l1v);
  for (uint32_t x = lane; x < K * C; x += 32) s_bins[warp][x] = 0.f;
  __syncthreads();
  float lv[K], l1v[K];
#pragma unroll
  for (uint32_t k = 0; k < K; ++k) { lv[k] = s_lv[k]; l1v[k] = s_l1v[k]; }
  float nll = 0.f, A[K], B[K];
#pragma unroll
  for (uint32_t k = 0; k < K; ++k) { A[k] = 0.f; B[k] = 0.f; }
  float* bins = s_bins[warp];
  // log pi and the bins are class-major ([c][k]): one vector access per site
  using VecK = typename KVec<K>::type;
  for (uint64_t base = i0 + (threadIdx.x & ~31u); base < i1; base += CAL_THREADS) {
    const uint64_t i = base + lane;
    const bool act = i < i1;
    int32_t c = -1;
    float g[K];
    if (act) {
      const float al = float(__ldg(a.alt + i)), dl = float(__ldg(a.depth + i));
      c = __ldg(a.cls + i);
      float t[K], tmax = -INFINITY;
      KVec<K>::load(s_logpi + c * K, t);
#pragma unroll
      for (uint32_t k = 0; k < K; ++k) {
        t[k] += al * lv[k] + (dl - al) * l1v[k];
        tmax = fmaxf(tmax, t[k]);
      }
      float se = 0.f;
#pragma unroll
      for (uint32_t k = 0; k < K; ++k) { g[k] = __expf(t[k] - tmax); se += g[k]; }
      const float inv = 1.f / se;
      nll -= tmax + __logf(se);
#pragma unroll
      for (uint32_t k = 0; k < K; ++k) { g[k] *= inv; A[k] += g[k] * al; B[k] += g[k] * (dl - al); }
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, c);
    if (act) {
      if ((peers & (peers - 1)) == 0) {              // the only lane with this class
        KVec<K>::add(bins + c * K, g);
      } else {                                         // shared class: sum in lane order
        float sum[K];
#pragma unroll
        for (uint32_t k = 0; k < K; ++k) sum[k] = 0.f;
        for (uint32_t m = peers; m; m &= m - 1) {
          const int src = __ffs(m) - 1;
#pragma unroll
          for (uint32_t k = 0; k < K; ++k) sum[k] += __shfl_sync(peers, g[k], src);
        }
        if (lane == uint32_t(__ffs(peers) - 1)) KVec<K>::add(bins + c * K, sum);
      }
    }
    __syncwarp();
    (void)sizeof(VecK);
  }
  // block partial: warp sums, then a compensated sum over the warps
  float* out = partial + uint64_t(chunk) * a.part_stride;
  {
    float vals[1 + 2 * K];
    vals[0] = nll;
#pragma unroll
    for (uint32_t k = 0; k < K; ++k) { vals[1 + k] = A[k]; vals[1 + K + k] = B[k]; }
#pragma unroll
    for (uint32_t q = 0; q < 1 + 2 * K; ++q) {
      float v = vals[q];
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) s_red[warp][q] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < 1 + 2 * K) {
    Neu t;
    for (uint32_t w = 0; w < CAL_WARPS; ++w) t.add(s_red[w][threadIdx.x]);
    out[threadIdx.x] = t.value();
  }
  for (uint32_t x = threadIdx.x; x < K * C; x += blockDim.x) {
    const uint32_t k = x / C, c = x % C;
    Neu t;
    for (uint32_t w = 0; w < CAL_WARPS; ++w) t.add(s_bins[w][c * K + k]);
    out[1 + 2 * K + x] = t.value();
  }
}

// one CTA per replicate: chunk partials -> NLL and gradient (-> Adam step)
__global__ void __launch_bounds__(CAL_THREADS) k_calib_epilogue(CalibArgs a, float* __restrict__ params,
                                                                const uint32_t* __restrict__ rep_first_chunk,
                                                                const float* __restrict__ partial,
                                                                float* __restrict__ nll_out,
                                                                float* __restrict__ grad_out, AdamArgs adam) {
  __shared__ float s_tot[1 + 2 * CAL_MAXK + CAL_MAXK * CAL_MAXC];
  __shared__ float s_M[CAL_MAXK * CAL_MAXC];
  __shared__ float s_w[CAL_MAXK * CAL_MAXJ];
  __shared__ float s_grad[CAL_MAXK + CAL_MAXK * CAL_MAXJ + 1];
  __shared__ float s_Gk[CAL_MAXK];
  const uint32_t r = a.rep0 + blockIdx.x;
  const uint32_t K = a.K, J = a.J, C = a.C, P = a.P;
  const uint32_t nval = 1 + 2 * K + K * C;
  const uint32_t c0 = rep_first_chunk[r], c1 = rep_first_chunk[r + 1];
  for (uint32_t x = threadIdx.x; x < nval; x += blockDim.x) {
    Neu t;
    for (uint32_t ch = c0; ch < c1; ++ch) t.add(partial[uint64_t(ch) * a.part_stride + x]);
    s_tot[x] = t.value();
  }
  float* p = params + uint64_t(r) * P;
  // exposures and mixtures
  for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
    const float* th = p + K + k * J;
    float mx = th[0];
    for (uint32_t j = 1; j < J; ++j) mx = fmaxf(mx, th[j]);
    float den = 0.f;
    for (uint32_t j = 0; j < J; ++j) den += expf(th[j] - mx);
    for (uint32_t j = 0; j < J; ++j) s_w[k * J + j] = expf(th[j] - mx) / den;
  }
  __syncthreads();
  for (uint32_t x = threadIdx.x; x < K * C; x += blockDim.x) {
    const uint32_t k = x / C, c = x % C;
    float m = 0.f;
    for (uint32_t j = 0; j < J; ++j) m += s_w[k * J + j] * a.sig[j * C + c];
    s_M[x] = fmaxf(m, 1e-30f);
  }
  if (threadIdx.x < K) {
    Neu g;
    for (uint32_t c = 0; c < C; ++c) g.add(s_tot[1 + 2 * K + threadIdx.x * C + c]);
    s_Gk[threadIdx.x] = g.value();
  }
  __syncthreads();
  const float* G = s_tot + 1 + 2 * K;
  if (threadIdx.x == 0) {
    // d/d lr_k = -G_k + N r_k L_k / Z   (N = sum_k G_k = number of sites)
    float Z = 0.f, N = 0.f;
    for (uint32_t k = 0; k < K; ++k) { Z += expf(p[k]) * a.epoch_w[r * K + k]; N += s_Gk[k]; }
    for (uint32_t k = 0; k < K; ++k) s_grad[k] = -s_Gk[k] + N * expf(p[k]) * a.epoch_w[r * K + k] / Z;
    // d/d rho = -(1 - sigma) sum_k (A_k - B_k v_k / (1 - v_k))
    const float sig = 1.f / (1.f + expf(-p[K + K * J]));
    float acc = 0.f;
    for (uint32_t k = 0; k < K; ++k) {
      const float v = sig * a.phi[r * K + k] * 0.5f;
      acc += s_tot[1 + k] - s_tot[1 + K + k] * v / (1.f - v);
    }
    s_grad[K + K * J] = -(1.f - sig) * acc;
  }
  // d/d theta_kj = -w_kj (sum_c G_k(c) S_j(c) / M_k(c) - G_k)
  for (uint32_t x = threadIdx.x; x < K * J; x += blockDim.x) {
    const uint32_t k = x / J, j = x % J;
    Neu s;
    for (uint32_t c = 0; c < C; ++c) s.add(G[k * C + c] * a.sig[j * C + c] / s_M[k * C + c]);
    s_grad[K + x] = -s_w[x] * (s.value() - s_Gk[k]);
  }
  __syncthreads();
  if (threadIdx.x == 0 && nll_out) nll_out[r] = s_tot[0];
  for (uint32_t q = threadIdx.x; q < P; q += blockDim.x) {
    const float g = s_grad[q];
    if (grad_out) grad_out[uint64_t(r) * P + q] = g;
    if (adam.m) {   // Adam step on the parameters (bias-corrected, step counter per replicate)
      const uint64_t o = uint64_t(r) * P + q;
      const float t = float(adam.step[r] + 1);
      const float m = adam.beta1 * adam.m[o] + (1.f - adam.beta1) * g;
      const float v = adam.beta2 * adam.v[o] + (1.f - adam.beta2) * g * g;
      adam.m[o] = m; adam.v[o] = v;
      const float mh = m / (1.f - powf(adam.beta1, t)), vh = v / (1.f - powf(adam.beta2, t));
      p[q] -= adam.lr * mh / (sqrtf(vh) + adam.eps);
    }
  }
  __syncthreads();
  if (adam.m && threadIdx.x == 0) adam.step[r] += 1;
}

void calib_launch(const CalibArgs& a, float* params, const uint32_t* chunk_rep, const uint64_t* chunk_start,
                  uint32_t n_chunks, const uint32_t* rep_first_chunk, uint32_t n_rep, float* partial, float* nll,
                  float* grad, const AdamArgs& adam, cudaStream_t st) {
  if (n_chunks) {
    switch (a.K) {
#define PG_CALIB_K(KK) case KK: k_calib_sites<KK><<<n_chunks, CAL_THREADS, 0, st>>>(a, params, chunk_rep, chunk_start, partial); break;
      PG_CALIB_K(1) PG_CALIB_K(2) PG_CALIB_K(3) PG_CALIB_K(4) PG_CALIB_K(5) PG_CALIB_K(6) PG_CALIB_K(7) PG_CALIB_K(8)
#undef PG_CALIB_K
    }
    note_launch();
  }
  if (n_rep) {
    k_calib_epilogue<<<n_rep, CAL_THREADS, 0, st>>>(a, params, rep_first_chunk, partial, nll, grad, adam);
    note_launch();
  }
}

}  // namespace pg
