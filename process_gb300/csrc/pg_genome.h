// Host-side replay of copy-number events into genotype classes.
//
// Reference semantics (ProCESS wrapper; RACES absent): driver CNAs and WGD
// are part of a mutant's driver list and are applied in declaration order
// with its SNVs/indels (src/mutation_engine.cpp:789-862,
// vignettes/mutations.Rmd:159-177); passenger CNAs are drawn from a
// candidate list (src/mutation_engine.cpp:441-487) at the species' CNA rate;
// with avoid_homozygous_losses a passenger deletion never removes the last
// allele of a region (src/mutation_engine.cpp:1356).
//
// Model restated here:
//   * a genome is a set of fragments (allele instance, [begin, end)) in
//     absolute coordinates; the germline has instances 0 and 1 over every
//     chromosome;
//   * amplification of [b, e) from instance X creates a new instance X' over
//     the part of [b, e) X covers; deletion removes [b, e) from X; WGD gives
//     every present instance a copy over all its fragments;
//   * the instance an event acts on is chosen among the instances covering
//     the region start (sorted by id): the given allele ordinal, or uniformly
//     with the event's Philox words; an event whose region start is not
//     covered does nothing;
//   * instance ids are assigned in event order (nodes in topological order,
//     events in application order), so they are canonical;
//   * every instance records its parent and the order key of the copy that
//     made it: (Euler preorder index of the edge << 16) | (event index + 1).
#pragma once
#include <algorithm>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <vector>

namespace pg {

struct Frag {
  uint32_t inst, b, e;   // absolute [b, e)
};

struct InstInfo {
  int32_t parent;        // -1 for the germline instances
  uint64_t key;          // order key of the copy that created it
};

using GenomeFrags = std::vector<Frag>;

// instances covering absolute position p, sorted by id
inline std::vector<uint32_t> covering_insts(const GenomeFrags& g, uint32_t p) {
  std::vector<uint32_t> out;
  for (const Frag& f : g)
    if (f.b <= p && p < f.e) out.push_back(f.inst);
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return out;
}

inline void frag_delete(GenomeFrags& g, uint32_t inst, uint32_t b, uint32_t e) {
  GenomeFrags out;
  for (const Frag& f : g) {
    if (f.inst != inst || f.e <= b || f.b >= e) { out.push_back(f); continue; }
    if (f.b < b) out.push_back({f.inst, f.b, b});
    if (f.e > e) out.push_back({f.inst, e, f.e});
  }
  g.swap(out);
}

inline void frag_amplify(GenomeFrags& g, uint32_t src, uint32_t dst, uint32_t b, uint32_t e) {
  GenomeFrags add;
  for (const Frag& f : g) {
    if (f.inst != src || f.e <= b || f.b >= e) continue;
    add.push_back({dst, std::max(f.b, b), std::min(f.e, e)});
  }
  g.insert(g.end(), add.begin(), add.end());
}

inline uint64_t frag_size(const GenomeFrags& g) {
  uint64_t s = 0;
  for (const Frag& f : g) s += f.e - f.b;
  return s;
}

// Segments of a class: maximal runs of positions covered by the same sorted
// instance list (positions with no instance are left out).
struct Segment {
  uint32_t b, e;
  std::vector<uint32_t> insts;
};

inline std::vector<Segment> segments_of(const GenomeFrags& g) {
  std::vector<std::pair<uint32_t, int64_t>> ev;   // (position, +/-(inst+1))
  for (const Frag& f : g) {
    if (f.b >= f.e) continue;
    ev.push_back({f.b, int64_t(f.inst) + 1});
    ev.push_back({f.e, -(int64_t(f.inst) + 1)});
  }
  std::sort(ev.begin(), ev.end());
  std::map<uint32_t, int> active;
  std::vector<Segment> out;
  size_t i = 0;
  while (i < ev.size()) {
    const uint32_t pos = ev[i].first;
    while (i < ev.size() && ev[i].first == pos) {
      const int64_t x = ev[i].second;
      const uint32_t inst = uint32_t((x > 0 ? x : -x) - 1);
      if (x > 0) active[inst] += 1;
      else if (--active[inst] == 0) active.erase(inst);
      ++i;
    }
    if (i >= ev.size()) break;
    const uint32_t next = ev[i].first;
    if (active.empty() || next == pos) continue;
    std::vector<uint32_t> insts;
    for (auto& kv : active) insts.push_back(kv.first);
    if (!out.empty() && out.back().e == pos && out.back().insts == insts) out.back().e = next;
    else out.push_back({pos, next, insts});
  }
  return out;
}

}  // namespace pg
