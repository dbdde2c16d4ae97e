// Engine inputs read from the reference's files: signature tables
// (Signature<SBSType|IDType>::read_from_stream, called from
// src/mutation_engine.cpp:389-397).  Included by pg_api.cpp.
//
// A signature table is tab-separated text: a header whose first column is
// "Type" and whose other columns name the signatures, then one row per
// mutation class: its label and one probability per signature.  Labels are
// COSMIC's: "A[C>A]A" (5' base, substitution of the pyrimidine, 3' base) for
// the 96 SBS classes, "1:Del:C:0" .. "5:Del:M:5" (size, Del/Ins, C/T/R/M,
// count) for the 83 ID classes.  Rows may come in any order; every class
// appears exactly once.

namespace {

int base_index(char c) {
  switch (c) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return -1;
  }
}

// SBS class of a label "X[Y>Z]W": sub * 16 + five * 4 + three, sub in
// C>A, C>G, C>T, T>A, T>C, T>G; -1 when the label is not one
int sbs_label_class(const std::string& s) {
  if (s.size() != 7 || s[1] != '[' || s[3] != '>' || s[5] != ']') return -1;
  const int five = base_index(s[0]), three = base_index(s[6]), ref = base_index(s[2]), alt = base_index(s[4]);
  if (five < 0 || three < 0 || ref < 0 || alt < 0 || ref == alt) return -1;
  int sub = -1;
  if (ref == 1) sub = alt == 0 ? 0 : alt == 2 ? 1 : 2;        // C>A C>G C>T
  else if (ref == 3) sub = alt == 0 ? 3 : alt == 1 ? 4 : 5;   // T>A T>C T>G
  if (sub < 0) return -1;
  return sub * 16 + five * 4 + three;
}

// ID83 class of a label "size:Del|Ins:C|T|R|M:count" in COSMIC order; -1
// when the label is not one
int id_label_class(const std::string& s) {
  const size_t a = s.find(':'), b = a == std::string::npos ? a : s.find(':', a + 1),
               c = b == std::string::npos ? b : s.find(':', b + 1);
  if (c == std::string::npos || s.find(':', c + 1) != std::string::npos) return -1;
  std::string sz = s.substr(0, a), kind = s.substr(a + 1, b - a - 1), what = s.substr(b + 1, c - b - 1),
              cnt = s.substr(c + 1);
  if (sz == "5+") sz = "5";          // some tables write the open-ended size and count as "5+"
  if (cnt == "5+") cnt = "5";
  if (sz.size() != 1 || cnt.size() != 1 || sz[0] < '1' || sz[0] > '5' || cnt[0] < '0' || cnt[0] > '5') return -1;
  const int l = sz[0] - '0', k = cnt[0] - '0';
  const bool del = kind == "Del", ins = kind == "Ins";
  if (!del && !ins) return -1;
  if (l == 1) {
    if (what != "C" && what != "T") return -1;
    return (ins ? 12 : 0) + (what == "T" ? 6 : 0) + k;
  }
  if (what == "R") return (ins ? 48 : 24) + (l - 2) * 6 + k;
  if (what == "M" && del) {                          // microhomology of k bases (5: 5 or more)
    const int off[4] = {0, 1, 3, 6};                 // first class of each size
    if (k < 1 || k > (l < 5 ? l - 1 : 5)) return -1;
    return 72 + off[l - 2] + k - 1;
  }
  return -1;
}

std::vector<std::string> split_tabs(const std::string& line) {
  std::vector<std::string> out;
  size_t at = 0;
  for (;;) {
    const size_t t = line.find('\t', at);
    out.push_back(line.substr(at, t == std::string::npos ? std::string::npos : t - at));
    if (t == std::string::npos) break;
    at = t + 1;
  }
  for (auto& f : out) {           // trailing spaces and carriage returns
    while (!f.empty() && (f.back() == '\r' || f.back() == ' ')) f.pop_back();
    size_t i = 0;
    while (i < f.size() && f[i] == ' ') ++i;
    f.erase(0, i);
  }
  return out;
}

// the table as names and [signature][class] probabilities
void parse_signature_table(std::istream& in, int type, std::vector<std::string>& names, std::vector<double>& probs) {
  const int NC = type == 0 ? 96 : 83;
  std::string line;
  if (!std::getline(in, line)) throw DomainError("empty signature table");
  const auto head = split_tabs(line);
  if (head.empty() || head[0] != "Type") throw DomainError("the signature table's first column must be \"Type\"");
  if (head.size() < 2) throw DomainError("the signature table has no signature column");
  names.assign(head.begin() + 1, head.end());
  for (const auto& n : names) if (n.empty()) throw DomainError("empty signature name in the table header");
  const size_t S = names.size();
  probs.assign(S * NC, 0.0);
  std::vector<char> seen(NC, 0);
  size_t row = 1;
  while (std::getline(in, line)) {
    ++row;
    if (line.empty() || line == "\r") continue;
    const auto f = split_tabs(line);
    if (f.size() != S + 1)
      throw DomainError("row " + std::to_string(row) + " of the signature table has " + std::to_string(f.size()) +
                        " columns, the header " + std::to_string(S + 1));
    const int c = type == 0 ? sbs_label_class(f[0]) : id_label_class(f[0]);
    if (c < 0) throw DomainError("unknown " + std::string(type == 0 ? "SBS" : "ID") + " class \"" + f[0] + "\"");
    if (seen[c]) throw DomainError("class \"" + f[0] + "\" appears twice in the signature table");
    seen[c] = 1;
    for (size_t j = 0; j < S; ++j) {
      char* end = nullptr;
      const double v = std::strtod(f[j + 1].c_str(), &end);
      if (end == f[j + 1].c_str() || *end != 0 || !std::isfinite(v) || v < 0)
        throw DomainError("row " + std::to_string(row) + ": \"" + f[j + 1] + "\" is not a probability");
      probs[j * NC + size_t(c)] = v;
    }
  }
  for (int c = 0; c < NC; ++c)
    if (!seen[c]) throw DomainError("the signature table lacks class " + std::to_string(c) + " of " + std::to_string(NC));
}

}  // namespace

extern "C" {

pg_status pg_signature_table_read(int type, const char* path, uint32_t* n_sigs, uint64_t* names_size, char* names,
                                  double* probs) {
  return guarded([&] {
    require(path != nullptr, "NULL argument");
    require(type == 0 || type == 1, "type must be 0 (SBS) or 1 (ID)");
    std::ifstream in(path);
    if (!in) throw DomainError(std::string("cannot read the signature table \"") + path + "\"");
    std::vector<std::string> nm;
    std::vector<double> pr;
    parse_signature_table(in, type, nm, pr);
    std::string packed;
    for (const auto& n : nm) { packed += n; packed.push_back(0); }
    if (n_sigs) *n_sigs = uint32_t(nm.size());
    if (names_size) *names_size = packed.size();
    if (names) std::memcpy(names, packed.data(), packed.size());
    if (probs) std::copy(pr.begin(), pr.end(), probs);
  });
}

pg_status pg_engine_load_signatures_tsv(pg_engine* e, int type, const char* path) {
  return guarded([&] {
    require(e && path, "NULL argument");
    require(type == 0 || type == 1, "type must be 0 (SBS) or 1 (ID)");
    std::ifstream in(path);
    if (!in) throw DomainError(std::string("cannot read the signature table \"") + path + "\"");
    std::vector<std::string> names;
    std::vector<double> probs;
    parse_signature_table(in, type, names, probs);
    check_status(pg_engine_set_signatures(e, type, uint32_t(names.size()), probs.data()));
    std::vector<const char*> cn;
    for (const auto& n : names) cn.push_back(n.c_str());
    check_status(pg_engine_set_signature_names(e, type, uint32_t(cn.size()), cn.data()));
  });
}

}  // extern "C"
