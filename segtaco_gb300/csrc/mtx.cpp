// mtx.cpp -- MatrixMarket coordinate files -> host CSR (segtaco_mtx_read).
//
// File format (NIST MatrixMarket exchange format): a banner
//   %%MatrixMarket matrix coordinate <field> <symmetry>
// (field: real | double | integer | pattern | complex; symmetry: general |
// symmetric | skew-symmetric | hermitian), comment lines starting with '%', a
// size line "rows cols entries", then one line "i j [value [imaginary]]" per
// entry with 1-based indices.
//
// Patterns:
//   SEGTACO_MTX_SEGTACO_PATTERN: the CSR segTACO's read_mtx_file builds
//     (ds.h:183-268): symmetric files have every off-diagonal (i, j) mirrored,
//     then the coordinates are sorted and duplicates dropped (general files are
//     sorted only, duplicates kept); the CSR is then filled from the sorted list
//     but only up to the header's entry count (ds.h:252-262), so a mirrored file
//     keeps its first `entries` coordinates in row order.  (segTACO reads past
//     its list when deduplication leaves fewer than `entries`; here the list
//     simply ends.)
//   otherwise (complete): symmetric, skew-symmetric and hermitian files are
//     mirrored (skew: negated), coordinates sorted, duplicates merged (values
//     summed).
// Values:
//   SEGTACO_MTX_VALUES_FILE    the file's values (real part; pattern files: 1)
//   SEGTACO_MTX_VALUES_SEGTACO {0, 0.1, 0.2} uniformly, the distribution of
//                              segTACO's fill_random (ds.h:270-274), but drawn
//                              from a seeded generator (splitmix64 of seed and
//                              position) so runs are reproducible
//   SEGTACO_MTX_VALUES_ONES    all ones
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

using namespace segtaco;

namespace {

struct Entry {
  long long key;  // row << 32 | col
  float val;
};

uint64_t splitmix64(uint64_t x) {
  // Steele, Lea, Flood: "Fast splittable pseudorandom number generators" (2014)
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}

std::string lower(std::string s) {
  for (auto &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// Reads the whole file; returns false if it cannot be opened.
bool slurp(const char *path, std::string *out) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out->append(buf, n);
  fclose(f);
  return true;
}

struct Cursor {
  const char *p, *end;
  int line = 1;
  bool at_end() const { return p >= end; }
  std::string getline() {
    const char *s = p;
    while (p < end && *p != '\n') ++p;
    std::string r(s, p);
    if (p < end) ++p;
    ++line;
    if (!r.empty() && r.back() == '\r') r.pop_back();
    return r;
  }
  void skip_space() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) {
      if (*p == '\n') ++line;
      ++p;
    }
  }
  bool read_ll(long long *v) {
    skip_space();
    if (p >= end) return false;
    char *e = nullptr;
    *v = strtoll(p, &e, 10);
    if (e == p) return false;
    p = e;
    return true;
  }
  bool read_double(double *v) {
    skip_space();
    if (p >= end) return false;
    char *e = nullptr;
    *v = strtod(p, &e);
    if (e == p) return false;
    p = e;
    return true;
  }
};

}  // namespace

extern "C" {

int segtaco_mtx_read(const char *path, uint32_t flags, int32_t values, uint64_t seed,
                     segtaco_host_csr *out) {
  if (!path || !out) return set_error(SEGTACO_EINVAL, "mtx: NULL argument");
  memset(out, 0, sizeof(*out));
  if (values < SEGTACO_MTX_VALUES_FILE || values > SEGTACO_MTX_VALUES_ONES)
    return set_error(SEGTACO_EINVAL, "mtx: unknown values mode %d", values);
  std::string text;
  if (!slurp(path, &text)) return set_error(SEGTACO_EINVAL, "mtx: cannot open %s", path);
  Cursor c{text.data(), text.data() + text.size()};
  // banner
  const std::string banner = lower(c.getline());
  char obj[64] = {0}, fmt[64] = {0}, field[64] = {0}, sym[64] = {0};
  if (sscanf(banner.c_str(), "%%%%matrixmarket %63s %63s %63s %63s", obj, fmt, field, sym) != 4)
    return set_error(SEGTACO_EINVAL, "mtx: %s: no MatrixMarket banner", path);
  if (std::string(obj) != "matrix")
    return set_error(SEGTACO_EUNSUPPORTED, "mtx: object '%s' is not a matrix", obj);
  if (std::string(fmt) != "coordinate")
    return set_error(SEGTACO_EUNSUPPORTED, "mtx: only coordinate (sparse) files, not '%s'", fmt);
  const std::string fld(field), sy(sym);
  const bool pattern = fld == "pattern";
  const bool complex = fld == "complex";
  if (!pattern && !complex && fld != "real" && fld != "double" && fld != "integer")
    return set_error(SEGTACO_EUNSUPPORTED, "mtx: field '%s'", field);
  if (sy != "general" && sy != "symmetric" && sy != "skew-symmetric" && sy != "hermitian")
    return set_error(SEGTACO_EUNSUPPORTED, "mtx: symmetry '%s'", sym);
  const bool seg = flags & SEGTACO_MTX_SEGTACO_PATTERN;
  // segTACO mirrors only files marked symmetric (mm_is_symmetric) and treats
  // the other symmetries as general; the complete reading mirrors all three.
  const bool mirror = seg ? sy == "symmetric" : sy != "general";
  const bool negate = !seg && sy == "skew-symmetric";
  const bool dedup = seg ? sy == "symmetric" : true;
  // comments, then the size line
  std::string line;
  do {
    if (c.at_end()) return set_error(SEGTACO_EINVAL, "mtx: %s: no size line", path);
    line = c.getline();
  } while (line.empty() || line[0] == '%');
  long long nrow = 0, ncol = 0, nent = 0;
  if (sscanf(line.c_str(), "%lld %lld %lld", &nrow, &ncol, &nent) != 3 || nrow < 0 || ncol < 0 ||
      nent < 0)
    return set_error(SEGTACO_EINVAL, "mtx: %s: bad size line '%s'", path, line.c_str());
  if (nrow > 0x7fffffffLL || ncol > 0x7fffffffLL || nent > 0x7fffffffLL)
    return set_error(SEGTACO_EUNSUPPORTED, "mtx: %s: dimensions exceed int32", path);
  std::vector<Entry> e;
  e.reserve((size_t)nent * (mirror ? 2 : 1));
  for (long long k = 0; k < nent; ++k) {
    long long i, j;
    double v = 1.0, im;
    if (!c.read_ll(&i) || !c.read_ll(&j))
      return set_error(SEGTACO_EINVAL, "mtx: %s: entry %lld of %lld missing", path, k + 1, nent);
    if (!pattern && !c.read_double(&v))
      return set_error(SEGTACO_EINVAL, "mtx: %s: entry %lld has no value", path, k + 1);
    if (complex && !c.read_double(&im))
      return set_error(SEGTACO_EINVAL, "mtx: %s: entry %lld has no imaginary part", path, k + 1);
    if (i < 1 || i > nrow || j < 1 || j > ncol)
      return set_error(SEGTACO_EINVAL, "mtx: %s: entry %lld (%lld, %lld) outside %lld x %lld",
                       path, k + 1, i, j, nrow, ncol);
    const long long r = i - 1, cc = j - 1;
    e.push_back({(r << 32) | cc, (float)v});
    if (mirror && r != cc) e.push_back({(cc << 32) | r, (float)(negate ? -v : v)});
  }
  std::stable_sort(e.begin(), e.end(), [](const Entry &a, const Entry &b) { return a.key < b.key; });
  std::vector<Entry> u;
  u.reserve(e.size());
  if (!dedup) {
    u.swap(e);  // segTACO: unmirrored files keep duplicates
  } else {
    for (size_t k = 0; k < e.size(); ++k) {
      if (!u.empty() && u.back().key == e[k].key) {
        if (!seg) u.back().val += e[k].val;  // complete: duplicates summed
      } else {
        u.push_back(e[k]);
      }
    }
  }
  if (seg && (long long)u.size() > nent) u.resize((size_t)nent);  // ds.h:252-262
  if (u.size() > 0x7fffffffULL)
    return set_error(SEGTACO_EUNSUPPORTED, "mtx: %s: more than 2^31 - 1 nonzeros", path);
  const long long nnz = (long long)u.size();
  int32_t *rp = static_cast<int32_t *>(malloc(sizeof(int32_t) * (size_t)(nrow + 1)));
  int32_t *col = static_cast<int32_t *>(malloc(sizeof(int32_t) * (size_t)std::max(1LL, nnz)));
  float *val = static_cast<float *>(malloc(sizeof(float) * (size_t)std::max(1LL, nnz)));
  if (!rp || !col || !val) {
    free(rp);
    free(col);
    free(val);
    return set_error(SEGTACO_ENOMEM, "mtx: host allocation failed");
  }
  long long pos = 0;
  rp[0] = 0;
  for (long long r = 0; r < nrow; ++r) {
    while (pos < nnz && (u[(size_t)pos].key >> 32) == r) {
      col[pos] = (int32_t)(u[(size_t)pos].key & 0xffffffffLL);
      const float fv = u[(size_t)pos].val;
      if (values == SEGTACO_MTX_VALUES_FILE)
        val[pos] = fv;
      else if (values == SEGTACO_MTX_VALUES_ONES)
        val[pos] = 1.0f;
      else
        val[pos] = (float)(splitmix64(seed ^ (0x5E67AC0ULL + (uint64_t)pos)) % 3) / 10.0f;
      ++pos;
    }
    rp[r + 1] = (int32_t)pos;
  }
  out->M = (int32_t)nrow;
  out->K = (int32_t)ncol;
  out->nnz = nnz;
  out->row_ptr = rp;
  out->col = col;
  out->vals = val;
  return SEGTACO_OK;
}

void segtaco_host_csr_free(segtaco_host_csr *csr) {
  if (!csr) return;
  free(csr->row_ptr);
  free(csr->col);
  free(csr->vals);
  memset(csr, 0, sizeof(*csr));
}

}  // extern "C"
