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
// Kernels: k_calib_tables (one CTA per replicate) derives the replicate's
// constants; k_calib_sites (one CTA per (replicate, chunk of sites))
// computes per-site log-likelihoods and responsibilities in FP32 with the
// mixture weights in registers and only the site class's signature row
// S(c) gathered from shared memory:
//   u_k = log(exp(lr_k) L_k / Z) + a log v_k + (d - a) log(1 - v_k)
//   e_k = exp(u_k - max u),  q_k = M_k(c) e_k,  s = sum_k q_k
//   gamma_k = q_k / s,  log-likelihood = max u + log s
// and reduces
//   G_k = sum_i gamma_ik,  A_k = sum gamma_ik a_i,  B_k = sum gamma_ik (d_i - a_i),
//   H_kj = sum_i gamma_ik S_j(c_i) / M_k(c_i) = sum_i e_ik S_j(c_i) / s_i,  NLL
// (H carries the class dependence of the exposure gradient, so no per-class
// bins are needed) with per-thread FP32 sums over the thread's sites in
// order, a fixed warp tree and a Neumaier-compensated sum over the warps;
// k_calib_epilogue (one CTA per replicate) adds the chunk partials in a fixed
// order (compensated) and applies the chain rule, optionally followed by an
// Adam step on the parameters.  Every sum has a fixed order: results are
// deterministic.
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

// Per-replicate constants, once per evaluation, in the replicate's row of
// a.tab: log(exp(lr_k) L_k / Z) (K), log v_k (K), log(1 - v_k) (K), then the
// exposures w_kj (K x J).
__global__ void __launch_bounds__(32) k_calib_tables(CalibArgs a, const float* __restrict__ params) {
  const uint32_t r = a.rep0 + blockIdx.x;
  const uint32_t K = a.K, J = a.J, k = threadIdx.x;
  const float* p = params + uint64_t(r) * a.P;
  float* row = a.tab + uint64_t(r) * a.tab_stride;
  float Z = 0.f;
  for (uint32_t q = 0; q < K; ++q) Z += expf(p[q]) * a.epoch_w[r * K + q];
  if (k >= K) return;
  const float sig = 1.f / (1.f + expf(-p[K + K * J]));
  const float v = sig * a.phi[r * K + k] * 0.5f;
  row[k] = p[k] + logf(a.epoch_w[r * K + k]) - logf(Z);
  row[K + k] = logf(v);
  row[2 * K + k] = log1pf(-v);
  const float* th = p + K + k * J;
  float mx = th[0];
  for (uint32_t j = 1; j < J; ++j) mx = fmaxf(mx, th[j]);
  float den = 0.f;
  for (uint32_t j = 0; j < J; ++j) den += expf(th[j] - mx);
  for (uint32_t j = 0; j < J; ++j) row[3 * K + k * J + j] = expf(th[j] - mx) / den;
}

// Per-site work: every thread takes sites i0 + tid, i0 + tid + 256, ...
// (coalesced, four sites' loads in flight at a time) and keeps plain FP32
// sums over its sites, in site order.  The signature rows in shared memory
// are JP floats (J rounded up to 4 or 8, zero beyond J).
// packed f32x2 arithmetic (two lanes of one 64-bit register pair, each
// rounded as the scalar operation)
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
// base-2 exponential and logarithm (the PTX approximate instructions, FTZ)
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
#define PG_F2OP(NAME, OP)                                                                                        \
  __device__ __forceinline__ float2 NAME(float2 a, float2 b) {                                                \
    float2 d;                                                                                                  \
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t" OP " rd, ra, rb;\n\t" \
        "mov.b64 {%0, %1}, rd;\n\t}"                                                                          \
        : "=f"(d.x), "=f"(d.y)                                                                                 \
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                                             \
    return d;                                                                                                  \
  }
PG_F2OP(f2mul, "mul.rn.f32x2")
PG_F2OP(f2add, "add.rn.f32x2")
#undef PG_F2OP

// CTAs per SM asked of the register allocator: the per-thread constants and
// sums take about 1 + 6K + 2KJ registers, plus K of per-site temporaries
// (4 CTAs, 64 registers, for the small shapes whose sums fit: 5% faster at
// K = 4, J = 3 than 3 CTAs)
constexpr uint32_t calib_min_blocks(uint32_t K, uint32_t J) {
  return (K + K % 2) * (J + 4) <= 28 && J <= 7 ? 4
         : 1 + 7 * K + 2 * K * J <= 53        ? 3
         : 1 + 7 * K + 2 * K * J <= 96        ? 2
                                              : 1;
}

template <uint32_t K, uint32_t J>
__global__ void __launch_bounds__(CAL_THREADS, calib_min_blocks(K, J)) k_calib_sites(
    CalibArgs a, const float* __restrict__ params, const uint32_t* __restrict__ chunk_rep,
    const uint64_t* __restrict__ chunk_start, float* __restrict__ partial) {
  constexpr uint32_t JP = J > 4 ? 8 : 4;
  constexpr uint32_t NV = 1 + 3 * K + K * J;   // nll, A, B, G, H
  constexpr uint32_t U = 4;
  __shared__ __align__(16) float s_sig[JP * CAL_MAXC];
  __shared__ float s_row[3 * CAL_MAXK + CAL_MAXK * CAL_MAXJ];
  __shared__ float s_red[CAL_WARPS][NV];
  const uint32_t chunk = a.chunk0 + blockIdx.x;
  const uint32_t r = chunk_rep[chunk];
  const uint64_t i0 = chunk_start[chunk];
  const uint64_t i1 = min(i0 + a.chunk, a.site_off[r + 1]);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t x = threadIdx.x; x < JP * a.C / 4; x += CAL_THREADS)
    reinterpret_cast<float4*>(s_sig)[x] = reinterpret_cast<const float4*>(a.sig_rows)[x];
  for (uint32_t x = threadIdx.x; x < 3 * K + K * J; x += CAL_THREADS) s_row[x] = a.tab[uint64_t(r) * a.tab_stride + x];
  __syncthreads();
  // epochs in pairs (packed f32x2 arithmetic); an odd K gets a padding
  // epoch of weight exp(-inf) = 0
  constexpr uint32_t KH = (K + 1) / 2;
  float2 cst[KH], dlv[KH], l1v[KH], w[J][KH];
  auto at = [&](uint32_t k, uint32_t off, float pad) { return k < K ? s_row[off + k] : pad; };
  // the log-domain terms in base 2 (ex2 / lg2 directly, the NLL scaled back by ln 2)
  constexpr float LOG2E = 1.4426950408889634f, LN2 = 0.6931471805599453f;
#pragma unroll
  for (uint32_t h = 0; h < KH; ++h) {
    cst[h] = make_float2(LOG2E * at(2 * h, 0, 0.f), at(2 * h + 1, 0, -INFINITY) * LOG2E);
    // u_k = cst_k + a log v_k + (d - a) log(1 - v_k) = cst_k + a dlv_k + d l1v_k
    l1v[h] = make_float2(LOG2E * at(2 * h, 2 * K, 0.f), LOG2E * at(2 * h + 1, 2 * K, 0.f));
    dlv[h] = make_float2(LOG2E * at(2 * h, K, 0.f) - l1v[h].x, LOG2E * at(2 * h + 1, K, 0.f) - l1v[h].y);
#pragma unroll
    for (uint32_t j = 0; j < J; ++j)
      w[j][h] = make_float2(s_row[3 * K + 2 * h * J + j], 2 * h + 1 < K ? s_row[3 * K + (2 * h + 1) * J + j] : 0.f);
  }
  float nll = 0.f;
  float2 A[KH], D[KH], G[KH], H[J][KH];   // D_k = sum gamma_ik d_i (B_k = D_k - A_k)
#pragma unroll
  for (uint32_t h = 0; h < KH; ++h) {
    A[h] = D[h] = G[h] = make_float2(0.f, 0.f);
#pragma unroll
    for (uint32_t j = 0; j < J; ++j) H[j][h] = make_float2(0.f, 0.f);
  }
  auto site = [&](float al, float dl, int32_t c) {
    float sg[JP];
#pragma unroll
    for (uint32_t j = 0; j < JP; j += 4) {
      const float4 x = *reinterpret_cast<const float4*>(s_sig + c * JP + j);
      sg[j] = x.x; sg[j + 1] = x.y; sg[j + 2] = x.z; sg[j + 3] = x.w;
    }
    const float2 al2 = make_float2(al, al), dl2 = make_float2(dl, dl);
    float2 u[KH], m[KH];
    float umax = -INFINITY;
#pragma unroll
    for (uint32_t h = 0; h < KH; ++h) {
      u[h] = f2fma(dl2, l1v[h], f2fma(al2, dlv[h], cst[h]));
      umax = fmaxf(umax, fmaxf(u[h].x, u[h].y));
      m[h] = f2mul(w[0][h], make_float2(sg[0], sg[0]));
#pragma unroll
      for (uint32_t j = 1; j < J; ++j) m[h] = f2fma(w[j][h], make_float2(sg[j], sg[j]), m[h]);
    }
    float2 e[KH], q[KH], s2;
    const float2 nmax = make_float2(-umax, -umax);
#pragma unroll
    for (uint32_t h = 0; h < KH; ++h) {
      const float2 z = f2add(u[h], nmax);
      e[h] = make_float2(ex2_approx(z.x), ex2_approx(z.y));
      q[h] = f2mul(m[h], e[h]);
      s2 = h ? f2add(s2, q[h]) : q[h];
    }
    // a class that no epoch's mixture can emit (every M_k(c) = 0) keeps a
    // finite, tiny sum
    const float sum = fmaxf(s2.x + s2.y, 1e-30f);
    const float inv = __fdividef(1.f, sum);
    nll -= umax + lg2_approx(sum);
    const float2 inv2 = make_float2(inv, inv);
#pragma unroll
    for (uint32_t h = 0; h < KH; ++h) {
      const float2 g = f2mul(q[h], inv2), r = f2mul(e[h], inv2);
      A[h] = f2fma(g, al2, A[h]);
      D[h] = f2fma(g, dl2, D[h]);
      G[h] = f2add(G[h], g);
#pragma unroll
      for (uint32_t j = 0; j < J; ++j) H[j][h] = f2fma(r, make_float2(sg[j], sg[j]), H[j][h]);
    }
  };
  auto site_at = [&](uint64_t x) { site(float(__ldg(a.alt + x)), float(__ldg(a.depth + x)), __ldg(a.cls + x)); };
  auto site4 = [&](const int4& x, const int4& y, const int4& z) {
    site(float(x.x), float(y.x), z.x); site(float(x.y), float(y.y), z.y);
    site(float(x.z), float(y.z), z.z); site(float(x.w), float(y.w), z.w);
  };
  const bool vec = ((reinterpret_cast<uintptr_t>(a.alt) | reinterpret_cast<uintptr_t>(a.depth) |
                     reinterpret_cast<uintptr_t>(a.cls)) & 15u) == 0;
  if (vec) {
    // four consecutive sites per 16-byte load of each column; the unaligned
    // head [i0, v0) and tail [v1, i1) (under four sites each) site by site
    const uint64_t v0 = min((i0 + 3) & ~uint64_t(3), i1), v1 = max(i1 & ~uint64_t(3), v0);
    if (threadIdx.x < v0 - i0) site_at(i0 + threadIdx.x);
    if (threadIdx.x < i1 - v1) site_at(v1 + threadIdx.x);
    const int4* a4 = reinterpret_cast<const int4*>(a.alt);
    const int4* d4 = reinterpret_cast<const int4*>(a.depth);
    const int4* c4 = reinterpret_cast<const int4*>(a.cls);
    const uint64_t q1 = v1 / 4;
    for (uint64_t q = v0 / 4 + threadIdx.x; q < q1; q += CAL_THREADS) site4(__ldg(a4 + q), __ldg(d4 + q), __ldg(c4 + q));
  } else {
    // columns not 16-byte aligned: U sites in flight per thread, strided
    uint64_t i = i0 + threadIdx.x;
    for (; i + (U - 1) * CAL_THREADS < i1; i += U * CAL_THREADS) {
      float al[U], dl[U];
      int32_t c[U];
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) {
        al[u] = float(__ldg(a.alt + i + u * CAL_THREADS));
        dl[u] = float(__ldg(a.depth + i + u * CAL_THREADS));
        c[u] = __ldg(a.cls + i + u * CAL_THREADS);
      }
#pragma unroll
      for (uint32_t u = 0; u < U; ++u) site(al[u], dl[u], c[u]);
    }
    for (; i < i1; i += CAL_THREADS) site(float(__ldg(a.alt + i)), float(__ldg(a.depth + i)), __ldg(a.cls + i));
  }
  // block partial: warp trees, then a compensated sum over the warps
  float acc[NV];
  acc[0] = nll * LN2;
#pragma unroll
  for (uint32_t k = 0; k < K; ++k) {
    const bool hi = k & 1;
    acc[1 + k] = hi ? A[k / 2].y : A[k / 2].x;
    acc[1 + K + k] = hi ? D[k / 2].y - A[k / 2].y : D[k / 2].x - A[k / 2].x;
    acc[1 + 2 * K + k] = hi ? G[k / 2].y : G[k / 2].x;
#pragma unroll
    for (uint32_t j = 0; j < J; ++j) acc[1 + 3 * K + k * J + j] = hi ? H[j][k / 2].y : H[j][k / 2].x;
  }
#pragma unroll
  for (uint32_t q = 0; q < NV; ++q) {
    float v = acc[q];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp][q] = v;
  }
  __syncthreads();
  // partial layout: nll, A_k, B_k, G_k, H_kj (j < J)
  float* out = partial + uint64_t(chunk) * a.part_stride;
  for (uint32_t x = threadIdx.x; x < NV; x += blockDim.x) {
    Neu t;
    for (uint32_t w = 0; w < CAL_WARPS; ++w) t.add(s_red[w][x]);
    out[x] = t.value();
  }
}

// one CTA per replicate: chunk partials -> NLL and gradient (-> Adam step)
__global__ void __launch_bounds__(CAL_THREADS) k_calib_epilogue(CalibArgs a, float* __restrict__ params,
                                                                const uint32_t* __restrict__ rep_first_chunk,
                                                                const float* __restrict__ partial,
                                                                float* __restrict__ nll_out,
                                                                float* __restrict__ grad_out, AdamArgs adam) {
  __shared__ float s_tot[1 + 3 * CAL_MAXK + CAL_MAXK * CAL_MAXJ];
  __shared__ float s_w[CAL_MAXK * CAL_MAXJ];
  __shared__ float s_grad[CAL_MAXK + CAL_MAXK * CAL_MAXJ + 1];
  const uint32_t r = a.rep0 + blockIdx.x;
  const uint32_t K = a.K, J = a.J, P = a.P;
  const uint32_t nval = 1 + 3 * K + K * J;
  const uint32_t c0 = rep_first_chunk[r], c1 = rep_first_chunk[r + 1];
  for (uint32_t x = threadIdx.x; x < nval; x += blockDim.x) {
    Neu t;
    for (uint32_t ch = c0; ch < c1; ++ch) t.add(partial[uint64_t(ch) * a.part_stride + x]);
    s_tot[x] = t.value();
  }
  float* p = params + uint64_t(r) * P;
  // exposures
  for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
    const float* th = p + K + k * J;
    float mx = th[0];
    for (uint32_t j = 1; j < J; ++j) mx = fmaxf(mx, th[j]);
    float den = 0.f;
    for (uint32_t j = 0; j < J; ++j) den += expf(th[j] - mx);
    for (uint32_t j = 0; j < J; ++j) s_w[k * J + j] = expf(th[j] - mx) / den;
  }
  __syncthreads();
  const float* G = s_tot + 1 + 2 * K;
  const float* H = s_tot + 1 + 3 * K;
  if (threadIdx.x == 0) {
    // d/d lr_k = -G_k + N r_k L_k / Z   (N = sum_k G_k = number of sites)
    float Z = 0.f, N = 0.f;
    for (uint32_t k = 0; k < K; ++k) { Z += expf(p[k]) * a.epoch_w[r * K + k]; N += G[k]; }
    for (uint32_t k = 0; k < K; ++k) s_grad[k] = -G[k] + N * expf(p[k]) * a.epoch_w[r * K + k] / Z;
    // d/d rho = -(1 - sigma) sum_k (A_k - B_k v_k / (1 - v_k))
    const float sig = 1.f / (1.f + expf(-p[K + K * J]));
    float acc = 0.f;
    for (uint32_t k = 0; k < K; ++k) {
      const float v = sig * a.phi[r * K + k] * 0.5f;
      acc += s_tot[1 + k] - s_tot[1 + K + k] * v / (1.f - v);
    }
    s_grad[K + K * J] = -(1.f - sig) * acc;
  }
  // d/d theta_kj = -w_kj (sum_i gamma_ik S_j(c_i) / M_k(c_i) - G_k) = -w_kj (H_kj - G_k)
  for (uint32_t x = threadIdx.x; x < K * J; x += blockDim.x) s_grad[K + x] = -s_w[x] * (H[x] - G[x / J]);
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
  if (n_rep) {
    k_calib_tables<<<n_rep, 32, 0, st>>>(a, params);
    note_launch();
  }
  if (n_chunks) {
    switch (a.K * 8 + a.J - 9) {
#define PG_CALIB_J(KK, JJ) \
  case KK * 8 + JJ - 9: k_calib_sites<KK, JJ><<<n_chunks, CAL_THREADS, 0, st>>>(a, params, chunk_rep, chunk_start, partial); break;
#define PG_CALIB_K(KK) PG_CALIB_J(KK, 1) PG_CALIB_J(KK, 2) PG_CALIB_J(KK, 3) PG_CALIB_J(KK, 4) \
                       PG_CALIB_J(KK, 5) PG_CALIB_J(KK, 6) PG_CALIB_J(KK, 7) PG_CALIB_J(KK, 8)
      PG_CALIB_K(1) PG_CALIB_K(2) PG_CALIB_K(3) PG_CALIB_K(4) PG_CALIB_K(5) PG_CALIB_K(6) PG_CALIB_K(7) PG_CALIB_K(8)
#undef PG_CALIB_J
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
