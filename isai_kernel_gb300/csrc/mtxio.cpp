// Host-side ingest: Matrix Market coordinate files to CSR, and a binary BSR
// file format for fast reload.  Plain C++ (no device code).
//
// read_matrix_market_to_csr (read_matrix.h:12) reads real "general" files
// only: it checks for the banner, skips '%' lines, reads the size line and
// nnz 1-based triples, sorts them by (row, col) and keeps duplicates.  This
// reader gives the same CSR for such files and also handles the header it
// ignores: "symmetric" / "hermitian" (real) files are expanded to both
// triangles, "skew-symmetric" ones with the mirrored value negated,
// "pattern" entries read as 1.0, "integer" values as doubles.  Entries are
// range-checked (the reference indexes out of bounds on a bad entry), blank
// lines between comments are skipped, and ties of the sort keep file order.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bilu_isai.h"

namespace {

struct Entry {
  int r, c;
  double v;
};

struct Header {
  bool pattern = false, symmetric = false, skew = false;
};

std::string lower(std::string s) {
  for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

bool read_file(const char* path, std::string& text) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, k);
  bool ok = !std::ferror(f);
  std::fclose(f);
  return ok;
}

// Parses the whole file; entries are already expanded (symmetric kinds) and
// 0-based.  *bad receives the failing entry index (0-based) or -1.
int parse(const char* path, int* m, int* n, std::vector<Entry>& out, long long* bad) {
  *bad = -1;
  std::string text;
  if (!path || !read_file(path, text)) return BILU_ERR_IO;
  size_t pos = 0;
  auto next_line = [&](std::string& line) {
    if (pos >= text.size()) return false;
    size_t e = text.find('\n', pos);
    if (e == std::string::npos) e = text.size();
    line.assign(text, pos, e - pos);
    if (!line.empty() && line.back() == '\r') line.pop_back();
    pos = e + 1;
    return true;
  };
  std::string line;
  if (!next_line(line) || line.find("MatrixMarket") == std::string::npos) return BILU_ERR_IO;
  Header h;
  {
    // %%MatrixMarket matrix <format> <field> <symmetry>
    char t[5][64] = {{0}};
    int nt = std::sscanf(line.c_str(), "%63s %63s %63s %63s %63s", t[0], t[1], t[2], t[3], t[4]);
    if (nt >= 3 && lower(t[2]) != "coordinate") return BILU_ERR_UNSUPPORTED;
    if (nt >= 4) {
      std::string field = lower(t[3]);
      if (field == "complex") return BILU_ERR_UNSUPPORTED;
      h.pattern = field == "pattern";
    }
    if (nt >= 5) {
      std::string sym = lower(t[4]);
      h.symmetric = sym == "symmetric" || sym == "hermitian" || sym == "skew-symmetric";
      h.skew = sym == "skew-symmetric";
    }
  }
  do {
    if (!next_line(line)) return BILU_ERR_IO;
  } while (line.empty() || line[0] == '%' ||
           line.find_first_not_of(" \t") == std::string::npos);
  long long mm = 0, nn = 0, nnz = 0;
  if (std::sscanf(line.c_str(), "%lld %lld %lld", &mm, &nn, &nnz) != 3 || mm < 0 || nn < 0 ||
      nnz < 0 || mm > INT32_MAX || nn > INT32_MAX)
    return BILU_ERR_IO;
  *m = (int)mm;
  *n = (int)nn;
  out.clear();
  out.reserve((size_t)nnz * (h.symmetric ? 2 : 1));
  const char* p = text.c_str() + std::min(pos, text.size());
  const char* end = text.c_str() + text.size();
  for (long long k = 0; k < nnz; ++k) {
    char* q = nullptr;
    errno = 0;
    long long r = std::strtoll(p, &q, 10);
    if (q == p) { *bad = k; return BILU_ERR_IO; }
    p = q;
    long long c = std::strtoll(p, &q, 10);
    if (q == p) { *bad = k; return BILU_ERR_IO; }
    p = q;
    double v = 1.0;
    if (!h.pattern) {
      v = std::strtod(p, &q);
      if (q == p) { *bad = k; return BILU_ERR_IO; }
      p = q;
    }
    if (r < 1 || r > mm || c < 1 || c > nn || p > end) { *bad = k; return BILU_ERR_IO; }
    out.push_back({(int)(r - 1), (int)(c - 1), v});
    if (h.symmetric && r != c) out.push_back({(int)(c - 1), (int)(r - 1), h.skew ? -v : v});
  }
  if (out.size() > (size_t)INT32_MAX) return BILU_ERR_UNSUPPORTED;
  std::stable_sort(out.begin(), out.end(), [](const Entry& a, const Entry& b) {
    return a.r != b.r ? a.r < b.r : a.c < b.c;
  });
  return BILU_OK;
}

// 64-bit FNV-1a over 8-byte words (the tail zero-padded), chained across
// the sections of the file.
uint64_t hash_words(const void* data, size_t bytes, uint64_t h) {
  const unsigned char* b = (const unsigned char*)data;
  size_t full = bytes / 8;
  for (size_t i = 0; i < full; ++i) {
    uint64_t w;
    std::memcpy(&w, b + 8 * i, 8);
    h = (h ^ w) * 1099511628211ull;
  }
  if (bytes % 8) {
    uint64_t w = 0;
    std::memcpy(&w, b + 8 * full, bytes % 8);
    h = (h ^ w) * 1099511628211ull;
  }
  return h;
}

constexpr char kMagic[8] = {'B', 'I', 'L', 'U', 'B', 'S', 'R', '1'};

struct FileHeader {
  char magic[8];
  int32_t bs;
  int32_t reserved;
  int64_t nb;
  int64_t nnzb;
  uint64_t checksum;  // over rowptr, colind, values
};
static_assert(sizeof(FileHeader) == 40, "header layout");

}  // namespace

extern "C" int bilu_mtx_read(const char* path, int* h_nrows, int* h_ncols, long long* h_nnz,
                             int* h_row, int* h_col, double* h_val, long long* h_bad_entry) {
  long long bad = -1;
  if (h_bad_entry) *h_bad_entry = -1;
  if (!h_nrows || !h_ncols || !h_nnz) return BILU_ERR_ARG;
  bool fill = h_row || h_col || h_val;
  if (fill && (!h_row || !h_col || !h_val)) return BILU_ERR_ARG;
  long long cap = *h_nnz;
  int m = 0, n = 0;
  std::vector<Entry> e;
  int rc = parse(path, &m, &n, e, &bad);
  if (h_bad_entry) *h_bad_entry = bad;
  if (rc != BILU_OK) return rc;
  *h_nrows = m;
  *h_ncols = n;
  *h_nnz = (long long)e.size();
  if (!fill) return BILU_OK;
  if (cap < (long long)e.size()) return BILU_ERR_WORKSPACE;
  std::fill(h_row, h_row + (size_t)m + 1, 0);
  for (const Entry& x : e) h_row[x.r + 1] += 1;
  for (int i = 0; i < m; ++i) h_row[i + 1] += h_row[i];
  for (size_t k = 0; k < e.size(); ++k) {
    h_col[k] = e[k].c;
    h_val[k] = e[k].v;
  }
  return BILU_OK;
}

extern "C" int bilu_bsr_save(const char* path, int nb, int nnzb, int bs, const int* h_row,
                             const int* h_col, const double* h_val) {
  if (!path || nb < 0 || nnzb < 0 || bs < 1 || !h_row || (nnzb > 0 && (!h_col || !h_val)))
    return BILU_ERR_ARG;
  if (h_row[0] != 0 || h_row[nb] != nnzb) return BILU_ERR_PATTERN;
  size_t nv = (size_t)nnzb * bs * bs;
  FileHeader hd{};
  std::memcpy(hd.magic, kMagic, 8);
  hd.bs = bs;
  hd.nb = nb;
  hd.nnzb = nnzb;
  uint64_t h = 1469598103934665603ull;
  h = hash_words(h_row, sizeof(int) * ((size_t)nb + 1), h);
  h = hash_words(h_col, sizeof(int) * (size_t)nnzb, h);
  h = hash_words(h_val, sizeof(double) * nv, h);
  hd.checksum = h;
  FILE* f = std::fopen(path, "wb");
  if (!f) return BILU_ERR_IO;
  bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 &&
            std::fwrite(h_row, sizeof(int), (size_t)nb + 1, f) == (size_t)nb + 1 &&
            std::fwrite(h_col, sizeof(int), (size_t)nnzb, f) == (size_t)nnzb &&
            std::fwrite(h_val, sizeof(double), nv, f) == nv;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BILU_OK : BILU_ERR_IO;
}

extern "C" int bilu_bsr_load(const char* path, int* h_nb, int* h_nnzb, int* h_bs, int* h_row,
                             int* h_col, double* h_val) {
  if (!path || !h_nb || !h_nnzb || !h_bs) return BILU_ERR_ARG;
  bool fill = h_row || h_col || h_val;
  if (fill && (!h_row || !h_col || !h_val)) return BILU_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return BILU_ERR_IO;
  FileHeader hd{};
  int rc = BILU_OK;
  if (std::fread(&hd, sizeof(hd), 1, f) != 1 || std::memcmp(hd.magic, kMagic, 8) != 0 ||
      hd.bs < 1 || hd.bs > 64 || hd.nb < 0 || hd.nb > INT32_MAX || hd.nnzb < 0 ||
      hd.nnzb > INT32_MAX)
    rc = BILU_ERR_IO;
  if (rc == BILU_OK && fill) {
    if (hd.nb != *h_nb || hd.nnzb != *h_nnzb || hd.bs != *h_bs) {
      rc = BILU_ERR_ARG;  // buffers sized for another file
    } else {
      size_t nv = (size_t)hd.nnzb * hd.bs * hd.bs;
      bool ok = std::fread(h_row, sizeof(int), (size_t)hd.nb + 1, f) == (size_t)hd.nb + 1 &&
                std::fread(h_col, sizeof(int), (size_t)hd.nnzb, f) == (size_t)hd.nnzb &&
                std::fread(h_val, sizeof(double), nv, f) == nv;
      if (!ok) {
        rc = BILU_ERR_IO;
      } else {
        uint64_t h = 1469598103934665603ull;
        h = hash_words(h_row, sizeof(int) * ((size_t)hd.nb + 1), h);
        h = hash_words(h_col, sizeof(int) * (size_t)hd.nnzb, h);
        h = hash_words(h_val, sizeof(double) * nv, h);
        if (h != hd.checksum) rc = BILU_ERR_IO;
      }
      if (rc == BILU_OK) {
        // structural check: monotone row pointers, columns in range
        if (h_row[0] != 0 || h_row[hd.nb] != hd.nnzb) rc = BILU_ERR_PATTERN;
        for (long long i = 0; rc == BILU_OK && i < hd.nb; ++i)
          if (h_row[i + 1] < h_row[i]) rc = BILU_ERR_PATTERN;
        for (long long k = 0; rc == BILU_OK && k < hd.nnzb; ++k)
          if (h_col[k] < 0 || h_col[k] >= hd.nb) rc = BILU_ERR_PATTERN;
      }
    }
  }
  std::fclose(f);
  if (rc == BILU_OK || rc == BILU_ERR_PATTERN) {
    *h_nb = (int)hd.nb;
    *h_nnzb = (int)hd.nnzb;
    *h_bs = hd.bs;
  }
  return rc;
}
