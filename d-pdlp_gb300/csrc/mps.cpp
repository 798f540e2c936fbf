// mps.cpp -- free-format MPS reader (read_mps_file).
//
// Replaces the reference's reader (src/mps_parser.c:365-777) with the same
// reading of the format, including its conventions:
//   * tokens are separated by blanks or tabs; lines starting with '*' are
//     comments; a line with one alphabetic token is a section header (ROWS,
//     COLUMNS, RHS, RANGES, BOUNDS, OBJSENSE, ENDATA; NAME lines carry two
//     tokens and are skipped);
//   * the objective is the first N row, or the first row when there is none;
//     other N rows are dropped; E / L / G rows become constraints in order of
//     appearance with [rhs, rhs], (-inf, rhs], [rhs, +inf) and rhs 0 by
//     default;
//   * COLUMNS: a line with an odd token count starts (or continues) column
//     token[0] followed by (row, value) pairs; an even count continues the
//     current column; 'MARKER' lines are skipped; objective entries add up;
//     entries of unknown rows are ignored; columns are numbered by first
//     appearance, with bounds [0, +inf) and cost 0 by default;
//   * RHS pairs (after the set name): on the objective row they set the
//     objective constant to -value;
//   * RANGES: G rows get upper = rhs + |R|, L rows lower = rhs - |R|, E rows
//     upper = rhs + R (R >= 0) or lower = rhs + R (R < 0);
//   * BOUNDS: LO, UP, FX, FR, MI, PL, BV (value 0 when absent); other kinds
//     and unknown columns are ignored;
//   * OBJSENSE MAX / MAXIMIZE (on the line after the header) negates the
//     objective and its constant, so the problem is always a minimisation;
//   * the matrix goes to CSR keeping the entries' input order within a row,
//     duplicates included.
// Files ending in ".gz" are read through zlib where the library was built
// with it.
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <unordered_map>
#include <vector>

#ifdef PDLP_HAVE_ZLIB
#include <zlib.h>
#endif

#include "cupdlpx.h"

namespace {

class LineSource {
 public:
  bool open(const char *path) {
    size_t L = strlen(path);
    gz_ = L > 3 && strcmp(path + L - 3, ".gz") == 0;
    if (gz_) {
#ifdef PDLP_HAVE_ZLIB
      g_ = gzopen(path, "rb");
      return g_ != nullptr;
#else
      fprintf(stderr, "ERROR: %s: compiled without zlib, gzip files cannot be read\n", path);
      return false;
#endif
    }
    f_ = fopen(path, "r");
    return f_ != nullptr;
  }
  ~LineSource() {
    if (f_) fclose(f_);
#ifdef PDLP_HAVE_ZLIB
    if (g_) gzclose(g_);
#endif
  }
  // next line without its terminator; false at end of input
  bool next(std::string &line) {
    line.clear();
    for (;;) {
      int c = getc_();
      if (c < 0) return !line.empty();
      if (c == '\n') return true;
      line.push_back((char)c);
    }
  }

 private:
  int getc_() {
    if (pos_ >= len_) {
      len_ = 0;
      pos_ = 0;
      if (f_) len_ = fread(buf_, 1, sizeof(buf_), f_);
#ifdef PDLP_HAVE_ZLIB
      else if (g_) {
        int r = gzread(g_, buf_, sizeof(buf_));
        len_ = r > 0 ? (size_t)r : 0;
      }
#endif
      if (len_ == 0) return -1;
    }
    return (unsigned char)buf_[pos_++];
  }
  bool gz_ = false;
  FILE *f_ = nullptr;
#ifdef PDLP_HAVE_ZLIB
  gzFile g_ = nullptr;
#endif
  char buf_[1 << 16];
  size_t pos_ = 0, len_ = 0;
};

enum class Sec { None, Rows, Columns, Rhs, Ranges, Bounds, ObjSense, End };

struct Parser {
  // rows as declared (type, name) until ROWS closes
  std::vector<std::pair<char, std::string>> declared;
  bool rows_done = false;
  std::string obj_row;
  bool has_obj = false;
  std::unordered_map<std::string, int> row_of, col_of;
  std::vector<char> row_type;
  std::vector<double> lc, uc;
  std::vector<double> cost, lv, uv;
  std::vector<int> ei, ej;
  std::vector<double> ev;
  std::string cur_col;
  bool have_col = false;
  double obj_const = 0.0;
  bool maximize = false;

  void close_rows() {
    if (rows_done) return;
    rows_done = true;
    int obj = -1;
    for (size_t i = 0; i < declared.size(); ++i)
      if (declared[i].first == 'N') {
        obj = (int)i;
        break;
      }
    if (obj < 0 && !declared.empty()) obj = 0;
    if (obj >= 0) {
      obj_row = declared[obj].second;
      has_obj = true;
    }
    for (size_t i = 0; i < declared.size(); ++i) {
      if ((int)i == obj) continue;
      char t = declared[i].first;
      if (t != 'E' && t != 'L' && t != 'G') continue;
      int idx = (int)row_type.size();
      // a repeated name keeps its first row, as a name map would
      if (!row_of.emplace(declared[i].second, idx).second) continue;
      row_type.push_back(t);
      lc.push_back(t == 'L' ? -INFINITY : 0.0);
      uc.push_back(t == 'G' ? INFINITY : 0.0);
    }
  }

  int row_index(const char *name) const {
    auto it = row_of.find(name);
    return it == row_of.end() ? -1 : it->second;
  }

  int column(const std::string &name) {
    auto it = col_of.find(name);
    if (it != col_of.end()) return it->second;
    int j = (int)cost.size();
    col_of.emplace(name, j);
    cost.push_back(0.0);
    lv.push_back(0.0);
    uv.push_back(INFINITY);
    return j;
  }

  bool is_obj(const char *name) const { return has_obj && obj_row == name; }

  bool line(Sec sec, char **tok, int nt) {
    switch (sec) {
      case Sec::ObjSense:
        if (!strcmp(tok[0], "MAX") || !strcmp(tok[0], "MAXIMIZE")) maximize = true;
        return true;
      case Sec::Rows:
        if (nt >= 2) declared.emplace_back(tok[0][0], tok[1]);
        return true;
      case Sec::Columns: {
        if (nt < 2 || !strcmp(tok[1], "'MARKER'")) return true;
        int first = 0;
        if (nt % 2) {
          cur_col = tok[0];
          have_col = true;
          first = 1;
        } else if (!have_col) {
          fprintf(stderr, "ERROR: MPS column entries before any column name\n");
          return false;
        }
        const int j = column(cur_col);
        for (int k = first; k + 1 < nt; k += 2) {
          const double v = atof(tok[k + 1]);
          if (is_obj(tok[k])) {
            cost[j] += v;
          } else {
            int i = row_index(tok[k]);
            if (i >= 0) {
              ei.push_back(i);
              ej.push_back(j);
              ev.push_back(v);
            }
          }
        }
        return true;
      }
      case Sec::Rhs:
        for (int k = 1; k + 1 < nt; k += 2) {
          const double v = atof(tok[k + 1]);
          if (is_obj(tok[k])) {
            obj_const = -v;
            continue;
          }
          int i = row_index(tok[k]);
          if (i < 0) continue;
          if (row_type[i] == 'L') uc[i] = v;
          else if (row_type[i] == 'G') lc[i] = v;
          else lc[i] = uc[i] = v;
        }
        return true;
      case Sec::Ranges:
        for (int k = 1; k + 1 < nt; k += 2) {
          int i = row_index(tok[k]);
          if (i < 0) continue;
          const double r = atof(tok[k + 1]);
          const char t = row_type[i];
          const double rhs = t == 'L' ? uc[i] : lc[i];
          if (t == 'G') uc[i] = rhs + fabs(r);
          else if (t == 'L') lc[i] = rhs - fabs(r);
          else if (r >= 0) uc[i] = rhs + r;
          else lc[i] = rhs + r;
        }
        return true;
      case Sec::Bounds: {
        if (nt < 3) return true;
        auto it = col_of.find(tok[2]);
        if (it == col_of.end()) return true;
        const int j = it->second;
        const double v = nt > 3 ? atof(tok[3]) : 0.0;
        const char *b = tok[0];
        if (!strcmp(b, "LO")) lv[j] = v;
        else if (!strcmp(b, "UP")) uv[j] = v;
        else if (!strcmp(b, "FX")) lv[j] = uv[j] = v;
        else if (!strcmp(b, "FR")) {
          lv[j] = -INFINITY;
          uv[j] = INFINITY;
        } else if (!strcmp(b, "MI")) lv[j] = -INFINITY;
        else if (!strcmp(b, "PL")) uv[j] = INFINITY;
        else if (!strcmp(b, "BV")) {
          lv[j] = 0.0;
          uv[j] = 1.0;
        }
        return true;
      }
      default:
        return true;
    }
  }
};

Sec header(const char *t) {
  if (!strcmp(t, "ROWS")) return Sec::Rows;
  if (!strcmp(t, "COLUMNS")) return Sec::Columns;
  if (!strcmp(t, "RHS")) return Sec::Rhs;
  if (!strcmp(t, "RANGES")) return Sec::Ranges;
  if (!strcmp(t, "BOUNDS")) return Sec::Bounds;
  if (!strcmp(t, "OBJSENSE")) return Sec::ObjSense;
  if (!strcmp(t, "ENDATA")) return Sec::End;
  return Sec::None;
}

}  // namespace

extern "C" lp_problem_t *read_mps_file(const char *filename) {
  if (!filename) return nullptr;
  LineSource src;
  if (!src.open(filename)) {
    fprintf(stderr, "ERROR: Could not open file %s\n", filename);
    return nullptr;
  }
  Parser P;
  Sec sec = Sec::None;
  std::string line;
  std::vector<char> buf;
  while (src.next(line)) {
    if (line.empty() || line[0] == '*' || line[0] == '\r') continue;
    buf.assign(line.begin(), line.end());
    buf.push_back('\0');
    char *tok[6];
    int nt = 0;
    char *save = nullptr;
    for (char *t = strtok_r(buf.data(), " \t\r\n", &save); t && nt < 6;
         t = strtok_r(nullptr, " \t\r\n", &save))
      tok[nt++] = t;
    if (nt == 0) continue;
    if (nt == 1 && isalpha((unsigned char)tok[0][0])) {
      Sec next = header(tok[0]);
      if (sec == Sec::Rows && next != Sec::Rows) P.close_rows();
      sec = next;
      if (sec == Sec::End) break;
      continue;
    }
    if (!P.line(sec, tok, nt)) {
      fprintf(stderr, "ERROR: Failed to parse MPS file.\n");
      return nullptr;
    }
  }
  // rows become constraints when the ROWS section is left by a header
  const int m = (int)P.row_type.size(), n = (int)P.cost.size();
  const long long nnz = (long long)P.ev.size();
  if (nnz > 0x7fffffffLL) {
    fprintf(stderr, "ERROR: MPS matrix has more than 2^31-1 entries\n");
    return nullptr;
  }
  // CSR, entries of a row in input order
  std::vector<int> rp((size_t)m + 1, 0), cj((size_t)nnz);
  std::vector<double> vx((size_t)nnz);
  for (long long k = 0; k < nnz; ++k) rp[P.ei[k] + 1]++;
  for (int i = 0; i < m; ++i) rp[i + 1] += rp[i];
  std::vector<int> pos(rp.begin(), rp.end() - 1);
  for (long long k = 0; k < nnz; ++k) {
    int d = pos[P.ei[k]]++;
    cj[d] = P.ej[k];
    vx[d] = P.ev[k];
  }
  if (P.maximize)
    for (double &c : P.cost) c = -c;
  const double c0 = P.maximize ? -P.obj_const : P.obj_const;
  matrix_desc_t A{};
  A.m = m;
  A.n = n;
  A.fmt = matrix_csr;
  A.zero_tolerance = 0.0;
  A.data.csr.nnz = (int)nnz;
  A.data.csr.row_ptr = rp.data();
  A.data.csr.col_ind = cj.data();
  A.data.csr.vals = vx.data();
  return create_lp_problem(P.cost.data(), &A, P.lc.data(), P.uc.data(), P.lv.data(),
                           P.uv.data(), &c0);
}
