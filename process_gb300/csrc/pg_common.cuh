// Shared device-side definitions: genome access, class tables, error flags.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pg {

// ---------------------------------------------------------------- bases
// 2-bit codes A=0 C=1 G=2 T=3; complement is 3-b.  The genome is stored as
// one concatenation of all chromosomes, 16 bases per u32 word, base i in bits
// 2*(i%16).  Absolute positions are u32, as the reference's
// AbsGenotypePosition (src/mutation_engine.hpp:34).
constexpr uint32_t BASE_INVALID = 4;

__device__ __forceinline__ uint32_t base_at(const uint32_t* __restrict__ g, uint32_t p) {
  return (__ldg(g + (p >> 4)) >> ((p & 15u) * 2u)) & 3u;
}

// ---------------------------------------------------------------- SBS classes
// 96 SBS classes in COSMIC order: class = sub*16 + five*4 + three with
// sub in {C>A, C>G, C>T, T>A, T>C, T>G}.  32 pyrimidine-centred contexts:
// ctx = (centre==T ? 16 : 0) + five*4 + three.
constexpr int N_SBS = 96;
constexpr int N_CTX = 32;
constexpr int N_ID = 83;

__host__ __device__ inline int sbs_class_context(int cls) { return (cls >= 48 ? 16 : 0) + (cls & 15); }
__host__ __device__ inline uint32_t sbs_class_alt(int cls) {
  // alt base of the pyrimidine strand: C>A A, C>G G, C>T T, T>A A, T>C C, T>G G
  const uint32_t alts[6] = {0, 2, 3, 0, 1, 2};
  return alts[cls >> 4];
}

// context id of the trinucleotide (x, y, z) read on the forward strand,
// folded to the pyrimidine-centred strand.  Sets *fwd to whether the forward
// strand already has the pyrimidine at the centre.
__host__ __device__ inline int context_of(uint32_t x, uint32_t y, uint32_t z, bool* fwd) {
  if (y == 1u || y == 3u) { *fwd = true; return (y == 3u ? 16 : 0) + int(x * 4u + z); }
  *fwd = false;
  const uint32_t cy = 3u - y, cx = 3u - z, cz = 3u - x;
  return (cy == 3u ? 16 : 0) + int(cx * 4u + cz);
}

// ---------------------------------------------------------------- status
// Device-side error flags (OR-ed); the host turns them into status codes.
enum : uint32_t {
  ERR_NONE = 0,
  ERR_INFINITE_SITES = 1u << 0,   // no free locus found within the attempt cap
  ERR_EMPTY_CLASS = 1u << 1,      // a drawn class had no indexed positions
  ERR_CAPACITY = 1u << 2,         // an output buffer was too small
  ERR_NO_ALLELE = 1u << 3,        // no allele covers the drawn locus within the cap
};

// Mutation kinds and natures (output column "class" of the reference's
// PhylogeneticForest getters, src/phylogenetic_forest.cpp:323-351).
enum : uint8_t { KIND_SNV = 0, KIND_INDEL = 1 };
enum : uint8_t { NATURE_PASSENGER = 0, NATURE_DRIVER = 1, NATURE_PRENEOPLASTIC = 2, NATURE_GERMINAL = 3 };

constexpr uint32_t LOCUS_INVALID = 0xffffffffu;   // a drawn position no allele of the cell covers
// Order of a mutation among the events of its edge.  Copy events (CNA
// amplifications, WGD) at event index j have order j + 1 and drivers at event
// index j have order j, so a copy follows a driver exactly when its index is
// larger; passengers follow every event of their edge; preneoplastic
// mutations precede every event of the forest (their edge shares preorder
// index 0 with the first root).
constexpr uint16_t SEQ_PASSENGER = 0x7fff;
constexpr uint16_t SEQ_PRENEOPLASTIC = 0;
constexpr uint32_t SEQ_MAX_EVENTS = 0x7ffd;       // events per edge (orders 1..0x7ffe)

}  // namespace pg

#include "pg_kernels.h"

namespace pg {

// allele instances of genotype class `cls` covering absolute position `pos`:
// returns their number and sets *ioff (their first index in inst_list)
__device__ __forceinline__ uint32_t covering(const GenomeClasses& g, uint32_t cls, uint32_t pos, uint32_t* ioff) {
  const uint32_t b = __ldg(g.seg_off + cls), e = __ldg(g.seg_off + cls + 1);
  if (b == e) return 0;
  uint32_t lo = b, hi = e;                 // last segment starting at or before pos
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(g.seg_start + mid) <= pos) lo = mid; else hi = mid;
  }
  if (__ldg(g.seg_start + lo) <= pos && pos < __ldg(g.seg_end + lo)) {
    *ioff = __ldg(g.seg_ioff + lo);
    return __ldg(g.seg_icnt + lo);
  }
  return 0;
}

}  // namespace pg
