// Genome storage and the two site indices the placement kernels draw from.
//
// Reference behaviour (ProCESS wrapper, RACES internals absent):
//   * ContextIndex<uint32_t>::build_index(ref, regions_to_avoid, context_sampling)
//     (src/mutation_engine.cpp:211-275, call :260): positions of the reference
//     grouped by pyrimidine-centred trinucleotide context, one kept in every
//     `context_sampling` occurrences (default 100, src/mutations.cpp:945-949).
//   * RSIndex::build_index(ref, max_motif_size, max_repetition_storage)
//     (src/mutation_engine.cpp:289-359, call :344): positions of repeated
//     sequences per ID class, at most `max_repetition_storage` per class.
//
// Here both are position lists in HBM, u32 absolute positions sorted
// ascending within each class, built in two streaming passes over the 2-bit
// genome: (1) per 1024-base tile, per class counts; (2) after a scan over
// tiles, every warp walks its tile again and writes the positions whose rank
// within their class is a multiple of the class stride.  Ranks inside a
// 32-position step come from __match_any_sync, so the lists are in position
// order without any sort.
#include <mutex>

#include "pg_common.cuh"
#include "pg_rng.cuh"
#include "pg_scan.cuh"
#include "pg_kernels.h"

namespace pg {

constexpr int TILE = 1024;
constexpr int WIN_BEFORE = 8;
constexpr int WIN_AFTER = 40;
constexpr int WIN = TILE + WIN_BEFORE + WIN_AFTER;   // bytes per warp
constexpr int WARPS = 8;

// ------------------------------------------------------------ genome fill
__global__ void k_genome_synth(uint32_t* __restrict__ words, uint64_t G, uint64_t nwords,
                               Key key, uint32_t gc_thr) {
  const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  uint32_t out = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint64_t blk = w * 4 + q;               // Philox block = 4 bases
    const U4 r = philox(key.k0, key.k1, uint32_t(blk), uint32_t(blk >> 32), 0u, TAG_GENOME);
    const uint32_t rw[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint64_t i = blk * 4 + j;
      if (i < G) {
        const uint32_t u = rw[j];
        // GC with probability gc_thr/2^32, then C/G or A/T by the low bit
        const uint32_t b = (u < gc_thr) ? (1u + (u & 1u)) : ((u & 1u) ? 3u : 0u);
        out |= b << (2 * (q * 4 + j));
      }
    }
  }
  words[w] = out;
}

__global__ void k_genome_pack(uint32_t* __restrict__ words, const uint8_t* __restrict__ codes,
                              uint64_t G, uint64_t nwords) {
  const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  uint32_t out = 0;
  for (int j = 0; j < 16; ++j) {
    const uint64_t i = w * 16 + j;
    if (i < G) out |= uint32_t(codes[i] & 3u) << (2 * j);
  }
  words[w] = out;
}

// ------------------------------------------------------------ class families
// SBS: one family, the trinucleotide context of p (needs both neighbours in
// the same chromosome).
struct SbsFamilies {
  static constexpr int NF = 1;
  static constexpr int NC = N_CTX;
  static constexpr bool AVOIDABLE = true;    // positions of the regions to avoid are not indexed
  template <class Get>
  __device__ static void classes(Get get, uint32_t p, uint32_t cs, uint32_t ce, int* out) {
    out[0] = -1;
    if (p <= cs || p + 1 >= ce) return;
    const uint32_t x = get(p - 1), y = get(p), z = get(p + 1);
    if (x > 3u || y > 3u || z > 3u) return;          // an unknown base (N) in the context
    bool fwd;
    out[0] = context_of(x, y, z, &fwd);
  }
};

// ID83 (COSMIC order).  A position p (the first deleted base, or the base
// before which bases are inserted; p-1 is the anchor) belongs to at most one
// class per family:
//   F0  1-bp deletion at a homopolymer run start, run length 1..6+     (0-11)
//   F1  1-bp insertion at a run start, run length 1..5+               (12-23, idx 1-5)
//   F2  1-bp C/G insertion with no adjacent C/G                       (12)
//   F3  1-bp T/A insertion with no adjacent T/A                       (18)
//   F4-7  l=2..5 deletion of the unit starting a repeat tract: repeat
//         count r>=2 -> 24+(l-2)*6+min(r-1,5); r==1 -> microhomology
//         m = common prefix of the unit and the following l bases:
//         m==0 -> 24+(l-2)*6, else 72+off(l)+m-1
//   F8-11 l=2..5 insertion of one more unit at a tract start, r>=1   (48+(l-2)*6+min(r,5))
//   F12-15 l=2..5 insertion of l random bases at a run start          (48+(l-2)*6)
struct IdFamilies {
  static constexpr int NF = 16;
  static constexpr int NC = N_ID;
  static constexpr bool AVOIDABLE = false;
  template <class Get>
  __device__ static void classes(Get get, uint32_t p, uint32_t cs, uint32_t ce, int* out) {
#pragma unroll
    for (int f = 0; f < NF; ++f) out[f] = -1;
    if (p <= cs || p >= ce) return;
    const uint32_t b = get(p), prev = get(p - 1);
    if (b > 3u || prev > 3u) return;                 // the site or its anchor is unknown (N)
    int h = 1;
    while (h < 6 && get(p + h) == b) ++h;
    const bool runstart = prev != b;
    const bool pyrT = (b == 3u || b == 0u);
    if (runstart) {
      out[0] = (pyrT ? 6 : 0) + h - 1;
      out[1] = 12 + (pyrT ? 6 : 0) + (h < 5 ? h : 5);
#pragma unroll
      for (int l = 2; l <= 5; ++l) out[12 + l - 2] = 48 + (l - 2) * 6;
    }
    if (b != 1u && b != 2u && prev != 1u && prev != 2u) out[2] = 12;
    if (b != 0u && b != 3u && prev != 0u && prev != 3u) out[3] = 18;
    const int mh_off[4] = {0, 1, 3, 6};
#pragma unroll
    for (int l = 2; l <= 5; ++l) {
      bool valid = true;
      for (int i = 0; i < l; ++i) valid = valid && get(p + i) != BASE_INVALID;
      if (!valid) continue;
      if (p >= cs + uint32_t(l)) {
        bool same = true;
        for (int i = 0; i < l; ++i) same = same && get(p - l + i) == get(p + i);
        if (same) continue;                       // not the start of the tract
      }
      int r = 1;
      while (r < 6) {
        bool same = true;
        for (int i = 0; i < l; ++i) same = same && get(p + r * l + i) == get(p + i);
        if (!same) break;
        ++r;
      }
      if (r >= 2) {
        out[4 + l - 2] = 24 + (l - 2) * 6 + (r - 1 < 5 ? r - 1 : 5);
      } else {
        int m = 0;
        while (m < l && get(p + l + m) == get(p + m)) ++m;
        out[4 + l - 2] = (m == 0) ? 24 + (l - 2) * 6 : 72 + mh_off[l - 2] + m - 1;
      }
      out[8 + l - 2] = 48 + (l - 2) * 6 + (r < 5 ? r : 5);
    }
  }
};

// ------------------------------------------------------------ index passes
struct WarpWindow {
  uint8_t* s;      // WIN bytes
  uint32_t start;  // absolute position of s[0]
};

// unknown bases (N) are bits of nmask (NULL: none), one bit per position
__device__ __forceinline__ bool base_unknown(const uint32_t* __restrict__ nmask, uint32_t q) {
  return nmask && ((__ldg(nmask + (q >> 5)) >> (q & 31u)) & 1u);
}

__device__ __forceinline__ void load_window(const uint32_t* __restrict__ g, const uint32_t* __restrict__ nmask,
                                            uint64_t G, uint32_t tile_start, uint8_t* s, int lane) {
  const int64_t w0 = int64_t(tile_start) - WIN_BEFORE;
  for (int i = lane; i < WIN; i += 32) {
    const int64_t q = w0 + i;
    s[i] = (q >= 0 && uint64_t(q) < G && !base_unknown(nmask, uint32_t(q))) ? uint8_t(base_at(g, uint32_t(q)))
                                                                           : uint8_t(BASE_INVALID);
  }
  __syncwarp();
}

// mode 0: count; mode 1: emit positions
template <class F, int MODE>
__global__ void __launch_bounds__(256) k_index_pass(const uint32_t* __restrict__ g,
                                                    const uint32_t* __restrict__ nmask,
                                                    const uint32_t* __restrict__ amask, uint64_t G,
                                                    const uint32_t* __restrict__ chr_off, int n_chr,
                                                    uint32_t ntiles, uint32_t* __restrict__ cnt,
                                                    const uint32_t* __restrict__ stride,
                                                    const uint64_t* __restrict__ list_off,
                                                    const uint32_t* __restrict__ list_len,
                                                    uint32_t* __restrict__ lists) {
  __shared__ uint8_t s_win[WARPS][WIN];
  __shared__ uint32_t s_run[WARPS][F::NC];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t tile = blockIdx.x * WARPS + warp;
  if (tile >= ntiles) return;
  const uint32_t tile_start = tile * TILE;
  for (int k = lane; k < F::NC; k += 32)
    s_run[warp][k] = MODE == 0 ? 0u : cnt[uint64_t(k) * ntiles + tile];
  load_window(g, nmask, G, tile_start, s_win[warp], lane);
  // chromosome of the tile start
  int c = 0;
  {
    int lo = 0, hi = n_chr;            // largest c with chr_off[c] <= tile_start
    while (hi - lo > 1) { int mid = (lo + hi) >> 1; if (__ldg(chr_off + mid) <= tile_start) lo = mid; else hi = mid; }
    c = lo;
  }
  const uint8_t* s = s_win[warp];
  for (int step = 0; step < TILE / 32; ++step) {
    const uint32_t p = tile_start + step * 32 + lane;
    int cls[F::NF];
    if (p < G) {
      while (c + 1 < n_chr && p >= __ldg(chr_off + c + 1)) ++c;
      const uint32_t cs = __ldg(chr_off + c), ce = __ldg(chr_off + c + 1);
      auto get = [&](uint32_t q) -> uint32_t {
        return (q >= cs && q < ce) ? uint32_t(s[q - tile_start + WIN_BEFORE]) : BASE_INVALID;
      };
      F::classes(get, p, cs, ce, cls);
      if (F::AVOIDABLE && base_unknown(amask, p)) cls[0] = -1;   // inside a region to avoid
    } else {
#pragma unroll
      for (int f = 0; f < F::NF; ++f) cls[f] = -1;
    }
#pragma unroll
    for (int f = 0; f < F::NF; ++f) {
      const int k = cls[f];
      const uint32_t peers = __match_any_sync(0xffffffffu, k);
      if (k >= 0) {
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        const uint32_t leader = __ffs(peers) - 1;
        if (MODE == 1) {
          const uint32_t r = s_run[warp][k] + rank;
          const uint32_t sd = stride[k];
          if (r % sd == 0) {
            const uint32_t idx = r / sd;
            if (idx < list_len[k]) lists[list_off[k] + idx] = p;
          }
        }
        __syncwarp(peers);
        if (uint32_t(lane) == leader) s_run[warp][k] += __popc(peers);
      }
      __syncwarp();
    }
  }
  if (MODE == 0) {
    for (int k = lane; k < F::NC; k += 32) cnt[uint64_t(k) * ntiles + tile] = s_run[warp][k];
  }
}

// ------------------------------------------------------------ host side
void genome_synth(uint32_t* words, uint64_t G, uint64_t seed, double gc, cudaStream_t st) {
  const uint64_t nwords = (G + 15) / 16;
  double t = gc * 4294967296.0;
  uint32_t thr = t >= 4294967295.0 ? 0xffffffffu : uint32_t(t);
  k_genome_synth<<<unsigned((nwords + 255) / 256), 256, 0, st>>>(words, G, nwords, make_key(seed), thr); note_launch();
}

void genome_pack(uint32_t* words, const uint8_t* codes, uint64_t G, cudaStream_t st) {
  const uint64_t nwords = (G + 15) / 16;
  k_genome_pack<<<unsigned((nwords + 255) / 256), 256, 0, st>>>(words, codes, G, nwords); note_launch();
}

uint32_t index_num_tiles(uint64_t G) { return uint32_t((G + TILE - 1) / TILE); }

template <class F>
static void index_count_t(const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                          const uint32_t* chr_off, int n_chr, uint32_t* cnt, uint32_t* part, uint32_t* totals,
                          cudaStream_t st) {
  const uint32_t ntiles = index_num_tiles(G);
  k_index_pass<F, 0><<<(ntiles + WARPS - 1) / WARPS, 256, 0, st>>>(g, nmask, amask, G, chr_off, n_chr, ntiles, cnt,
                                                                  nullptr, nullptr, nullptr, nullptr); note_launch();
  scan_rows<uint32_t>(cnt, cnt, ntiles, F::NC, part, totals, st);
}

template <class F>
static void index_emit_t(const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                         const uint32_t* chr_off, int n_chr, const uint32_t* cnt_scanned, const uint32_t* stride,
                         const uint64_t* list_off, const uint32_t* list_len, uint32_t* lists, cudaStream_t st) {
  const uint32_t ntiles = index_num_tiles(G);
  k_index_pass<F, 1><<<(ntiles + WARPS - 1) / WARPS, 256, 0, st>>>(g, nmask, amask, G, chr_off, n_chr, ntiles,
                                                                  const_cast<uint32_t*>(cnt_scanned),
                                                                  stride, list_off, list_len, lists); note_launch();
}

void index_count(int which, const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                 const uint32_t* chr_off, int n_chr, uint32_t* cnt, uint32_t* part, uint32_t* totals, cudaStream_t st) {
  if (which == 0) index_count_t<SbsFamilies>(g, nmask, amask, G, chr_off, n_chr, cnt, part, totals, st);
  else index_count_t<IdFamilies>(g, nmask, nullptr, G, chr_off, n_chr, cnt, part, totals, st);
}

void index_emit(int which, const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                const uint32_t* chr_off, int n_chr, const uint32_t* cnt_scanned, const uint32_t* stride,
                const uint64_t* list_off, const uint32_t* list_len, uint32_t* lists, cudaStream_t st) {
  if (which == 0)
    index_emit_t<SbsFamilies>(g, nmask, amask, G, chr_off, n_chr, cnt_scanned, stride, list_off, list_len, lists, st);
  else
    index_emit_t<IdFamilies>(g, nmask, nullptr, G, chr_off, n_chr, cnt_scanned, stride, list_off, list_len, lists,
                             st);
}

// the positions of the regions to avoid as bits of mask ((G + 31) / 32 words,
// zeroed by the caller)
__global__ void k_avoid_mask(const uint32_t* __restrict__ pos, uint64_t n, uint32_t* __restrict__ mask) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) atomicOr(mask + (pos[i] >> 5), 1u << (pos[i] & 31u));
}

void genome_avoid_mask(const uint32_t* pos, uint64_t n, uint32_t* mask, cudaStream_t st) {
  if (n) { k_avoid_mask<<<unsigned((n + 255) / 256), 256, 0, st>>>(pos, n, mask); note_launch(); }
}

int index_num_classes(int which) { return which == 0 ? SbsFamilies::NC : IdFamilies::NC; }

// ------------------------------------------------------------ allocation-free class counts
// The count pass above writes one count per (class, tile) into a table the
// engine allocates.  This variant keeps that table in a fixed array of the
// library's own device memory, so that a caller who may not allocate device
// memory can still count the classes of a genome it holds.  The array is
// sized for genomes up to NOALLOC_MAX_TILES tiles of 1024 bases (8 Mbp);
// every GPU that loads the library holds it (2.7 MB) until the process ends.
static __device__ __align__(256) uint32_t g_noalloc_tile_counts[N_ID * NOALLOC_MAX_TILES];

// per-class sum of the tile counts (one block per class)
__global__ void k_class_totals(const uint32_t* __restrict__ cnt, uint32_t ntiles, uint64_t* __restrict__ totals) {
  __shared__ uint64_t s_part[8];
  const uint32_t k = blockIdx.x;
  uint64_t acc = 0;
  for (uint32_t t = threadIdx.x; t < ntiles; t += blockDim.x) acc += cnt[uint64_t(k) * ntiles + t];
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t tot = 0;
    for (int w = 0; w < 8; ++w) tot += s_part[w];
    totals[k] = tot;
  }
}

// device address of g_noalloc_tile_counts per device (host code cannot use
// the symbol itself: on the host it names a stand-in, not device memory).
// The address is looked up once per device and kept; a cudaDeviceReset
// invalidates it, so the entry point is not for use after a device reset.
static std::mutex g_noalloc_mu;
static uint32_t* g_noalloc_addr[64] = {};

const char* index_counts_noalloc(int which, const uint32_t* g, uint64_t G, const uint32_t* chr_off, int n_chr,
                                 uint64_t* totals, cudaStream_t st) {
  if (G == 0 || G > uint64_t(NOALLOC_MAX_TILES) * TILE) return "genome length must be in [1, 8388608] bases";
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return "no current CUDA device";
  uint32_t* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_tile_counts) != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return "cudaGetSymbolAddress failed for the library's count array";
      }
      g_noalloc_addr[dev] = static_cast<uint32_t*>(p);
    }
    scratch = g_noalloc_addr[dev];
  }
  const uint32_t ntiles = index_num_tiles(G);
  const int nc = index_num_classes(which);
  // an error left pending by earlier work on this thread is not this call's:
  // report it as such and leave it pending for its owner, launching nothing
  if (cudaPeekAtLastError() != cudaSuccess) return "a CUDA error from earlier work is pending; nothing was launched";
  // every (class, tile) entry is written by the count pass: nothing to clear
  if (which == 0)
    k_index_pass<SbsFamilies, 0><<<(ntiles + WARPS - 1) / WARPS, 256, 0, st>>>(g, nullptr, nullptr, G, chr_off, n_chr, ntiles,
                                                                              scratch,
                                                                              nullptr, nullptr, nullptr, nullptr);
  else
    k_index_pass<IdFamilies, 0><<<(ntiles + WARPS - 1) / WARPS, 256, 0, st>>>(g, nullptr, nullptr, G, chr_off, n_chr, ntiles,
                                                                             scratch,
                                                                             nullptr, nullptr, nullptr, nullptr);
  k_class_totals<<<nc, 256, 0, st>>>(scratch, ntiles, totals);
  note_launch(2);
  if (cudaGetLastError() != cudaSuccess) return "launch of the count kernels failed";
  return nullptr;
}

}  // namespace pg

namespace pg {

__global__ void k_gather_bases(const uint32_t* __restrict__ g, const uint32_t* __restrict__ nmask,
                               const uint32_t* __restrict__ pos, uint64_t n, uint64_t G, uint8_t* __restrict__ out) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = pos[i] < G && !base_unknown(nmask, pos[i]) ? uint8_t(base_at(g, pos[i])) : uint8_t(BASE_INVALID);
}

void genome_gather(const uint32_t* g, const uint32_t* nmask, uint64_t G, const uint32_t* pos, uint64_t n,
                   uint8_t* out, cudaStream_t st) {
  if (n) { k_gather_bases<<<unsigned((n + 255) / 256), 256, 0, st>>>(g, nmask, pos, n, G, out); note_launch(); }
}

// SID strings of placed mutations (the ref and alt columns of the result data
// frames): up to 8 characters each, 4 bits per character (A 1, C 2, G 3, N 4,
// T 5, the characters' alphabetical order; 0 ends the string), the first in
// the highest nibble, so that codes compare as the strings do.  An SNV is
// (reference base, alt base); an insertion (anchor, anchor + inserted bases);
// a deletion (anchor + deleted bases, anchor).
__device__ __forceinline__ uint32_t sid_char(const uint32_t* __restrict__ g, const uint32_t* __restrict__ nmask,
                                             uint64_t G, uint64_t p) {
  if (p >= G) p = G - 1;
  if (base_unknown(nmask, p)) return 4u;
  const uint32_t b = base_at(g, uint32_t(p));
  return b == 3u ? 5u : b + 1u;
}

__global__ void k_row_info(const uint32_t* __restrict__ locus, const uint32_t* __restrict__ aux,
                           const uint8_t* __restrict__ kind, const uint8_t* __restrict__ sig,
                           const uint8_t* __restrict__ nature, const uint32_t* __restrict__ rows, uint64_t n,
                           const uint32_t* __restrict__ g, const uint32_t* __restrict__ nmask, uint64_t G,
                           uint4* __restrict__ out) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t m = rows ? rows[i] : i;
  const uint32_t L = locus[m], a = aux[m], k = kind[m];
  const uint32_t anchor = sid_char(g, nmask, G, L) << 28;
  uint32_t ref = anchor, alt = anchor;
  if (k == 0) {
    const uint32_t b = a & 3u;
    alt = (b == 3u ? 5u : b + 1u) << 28;
  } else {
    const uint32_t l = (a >> 1) & 7u;
    for (uint32_t q = 0; q < l; ++q) {
      if (a & 1u) {
        const uint32_t b = (a >> (8 + 2 * q)) & 3u;
        alt |= (b == 3u ? 5u : b + 1u) << (24 - 4 * q);
      } else {
        ref |= sid_char(g, nmask, G, uint64_t(L) + 1 + q) << (24 - 4 * q);
      }
    }
  }
  out[i] = make_uint4(L, ref, alt, k | (uint32_t(sig[m]) << 8) | (uint32_t(nature[m]) << 16));
}

void row_info(const uint32_t* locus, const uint32_t* aux, const uint8_t* kind, const uint8_t* sig,
              const uint8_t* nature, const uint32_t* rows, uint64_t n, const uint32_t* g, const uint32_t* nmask,
              uint64_t G, uint4* out, cudaStream_t st) {
  if (n) {
    k_row_info<<<unsigned((n + 255) / 256), 256, 0, st>>>(locus, aux, kind, sig, nature, rows, n, g, nmask, G, out);
    note_launch();
  }
}

// the unknown bases (codes > 3) of an uploaded genome as one bit per position,
// and whether there is any
__global__ void k_genome_nmask(const uint8_t* __restrict__ codes, uint64_t G, uint64_t nwords,
                               uint32_t* __restrict__ mask, uint32_t* __restrict__ any) {
  const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  uint32_t m = 0;
  for (int j = 0; j < 32; ++j) {
    const uint64_t i = w * 32 + j;
    if (i < G && codes[i] > 3u) m |= 1u << j;
  }
  mask[w] = m;
  if (m) atomicOr(any, 1u);
}

void genome_nmask(const uint8_t* codes, uint64_t G, uint32_t* mask, uint32_t* any, cudaStream_t st) {
  const uint64_t nwords = (G + 31) / 32;
  if (nwords) { k_genome_nmask<<<unsigned((nwords + 255) / 256), 256, 0, st>>>(codes, G, nwords, mask, any); note_launch(); }
}

}  // namespace pg
