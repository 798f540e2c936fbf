// lpgen.cpp -- seeded synthetic LPs for benchmarks and tests.
//
// Randomness is SplitMix64; the only transcendental functions (log for the
// normal draws, pow for the Zipf degrees) are evaluated with plain IEEE
// arithmetic below, and this file is compiled without floating-point
// contraction, so every host (x86 or Arm) generates bit-identical problems.
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <unordered_set>
#include <vector>

#include "cupdlpx.h"
#include "pdlp_gb300.h"

namespace {

struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  uint64_t below(uint64_t n) { return n ? next() % n : 0; }
  double normal();
};

const double kLn2Hi = 6.93147180369123816490e-01;
const double kLn2Lo = 1.90821492927058770002e-10;

// ln(x), x > 0 finite: x = f 2^e with f in [sqrt(1/2), sqrt(2)),
// ln f = 2 atanh(z), z = (f-1)/(f+1), odd series to z^31 (|z| <= 0.1716).
double det_log(double x) {
  int e;
  double f = frexp(x, &e);  // f in [0.5, 1)
  if (f < 0.70710678118654752440) {
    f *= 2.0;
    e -= 1;
  }
  double z = (f - 1.0) / (f + 1.0);
  double z2 = z * z;
  double term = z, s = 0.0;
  for (int k = 1; k <= 31; k += 2) {
    s += term / k;
    term *= z2;
  }
  return 2.0 * s + e * kLn2Lo + e * kLn2Hi;
}

// exp(y), |y| < 700: y = k ln2 + r, Taylor series of e^r to r^24.
double det_exp(double y) {
  double kf = floor(y / (kLn2Hi + kLn2Lo) + 0.5);
  double r = (y - kf * kLn2Hi) - kf * kLn2Lo;
  double term = 1.0, s = 1.0;
  for (int i = 1; i <= 24; ++i) {
    term = term * r / i;
    s += term;
  }
  return ldexp(s, (int)kf);
}

double Rng::normal() {  // Marsaglia polar method, one draw per call
  for (;;) {
    double u = 2.0 * uniform() - 1.0, v = 2.0 * uniform() - 1.0;
    double q = u * u + v * v;
    if (q > 0.0 && q < 1.0) return u * sqrt(-2.0 * det_log(q) / q);
  }
}

// Frees a problem made by alloc_problem (the arrays and the struct, as
// lp_problem_free does), so this file needs nothing else of the library.
void free_problem(lp_problem_t *p) {
  free(p->constraint_matrix_row_pointers);
  free(p->constraint_matrix_col_indices);
  free(p->constraint_matrix_values);
  free(p->objective_vector);
  free(p->variable_lower_bound);
  free(p->variable_upper_bound);
  free(p->constraint_lower_bound);
  free(p->constraint_upper_bound);
  free(p);
}

lp_problem_t *alloc_problem(int m, int n, long nnz) {
  lp_problem_t *p = (lp_problem_t *)calloc(1, sizeof(lp_problem_t));
  if (!p) return nullptr;
  p->num_constraints = m;
  p->num_variables = n;
  p->constraint_matrix_num_nonzeros = (int)nnz;
  p->constraint_matrix_row_pointers = (int *)malloc(sizeof(int) * ((size_t)m + 1));
  p->constraint_matrix_col_indices = (int *)malloc(sizeof(int) * (size_t)(nnz ? nnz : 1));
  p->constraint_matrix_values = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
  p->objective_vector = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
  p->variable_lower_bound = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
  p->variable_upper_bound = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
  p->constraint_lower_bound = (double *)malloc(sizeof(double) * (size_t)(m ? m : 1));
  p->constraint_upper_bound = (double *)malloc(sizeof(double) * (size_t)(m ? m : 1));
  if (!p->constraint_matrix_row_pointers || !p->constraint_matrix_col_indices ||
      !p->constraint_matrix_values || !p->objective_vector || !p->variable_lower_bound ||
      !p->variable_upper_bound || !p->constraint_lower_bound || !p->constraint_upper_bound) {
    free_problem(p);
    return nullptr;
  }
  return p;
}

// Entries given column by column (cols ascending, rows arbitrary within a
// column) -> CSR with ascending columns in each row (counting sort by row).
void coo_cols_to_csr(lp_problem_t *p, const std::vector<int> &ri, const std::vector<int> &ci,
                     const std::vector<double> &v) {
  const int m = p->num_constraints;
  int *rp = p->constraint_matrix_row_pointers;
  std::fill(rp, rp + m + 1, 0);
  for (int r : ri) rp[r + 1]++;
  for (int i = 0; i < m; ++i) rp[i + 1] += rp[i];
  std::vector<int> next(rp, rp + m);
  for (size_t k = 0; k < ri.size(); ++k) {
    int pos = next[ri[k]]++;
    p->constraint_matrix_col_indices[pos] = ci[k];
    p->constraint_matrix_values[pos] = v[k];
  }
}

// x0 ~ U[0,1]^n; 30% equality rows l = u = A x0, else l = A x0 - U[0,1],
// u = +inf; 0 <= x <= 10; c ~ U[-1,1]   (the bound rule of the configs)
void feasible_bounds(lp_problem_t *p, Rng &rng) {
  const int m = p->num_constraints, n = p->num_variables;
  std::vector<double> x0(n);
  for (int j = 0; j < n; ++j) x0[j] = rng.uniform();
  for (int i = 0; i < m; ++i) {
    double ax = 0.0;
    for (int k = p->constraint_matrix_row_pointers[i]; k < p->constraint_matrix_row_pointers[i + 1]; ++k)
      ax += p->constraint_matrix_values[k] * x0[p->constraint_matrix_col_indices[k]];
    if (rng.uniform() < 0.3) {
      p->constraint_lower_bound[i] = ax;
      p->constraint_upper_bound[i] = ax;
    } else {
      p->constraint_lower_bound[i] = ax - rng.uniform();
      p->constraint_upper_bound[i] = INFINITY;
    }
  }
  for (int j = 0; j < n; ++j) {
    p->variable_lower_bound[j] = 0.0;
    p->variable_upper_bound[j] = 10.0;
    p->objective_vector[j] = 2.0 * rng.uniform() - 1.0;
  }
  p->objective_constant = 0.0;
}

}  // namespace

extern "C" {

lp_problem_t *pdlp_generate_random_lp(int m, int n, long long nnz, unsigned long long seed) {
  if (m <= 0 || n <= 0 || nnz < 0 || nnz > (long long)m * n || nnz > 2000000000LL) return nullptr;
  Rng rng(seed);
  // distinct uniform positions, drawn column-major so the CSR build is stable
  std::unordered_set<uint64_t> seen;
  seen.reserve((size_t)nnz * 2);
  std::vector<uint64_t> keys;
  keys.reserve((size_t)nnz);
  while ((long long)keys.size() < nnz) {
    uint64_t i = rng.below((uint64_t)m), j = rng.below((uint64_t)n);
    uint64_t key = j * (uint64_t)m + i;
    if (seen.insert(key).second) keys.push_back(key);
  }
  std::vector<double> vals(keys.size());
  for (size_t k = 0; k < keys.size(); ++k) vals[k] = rng.normal();
  std::vector<size_t> order(keys.size());
  for (size_t k = 0; k < order.size(); ++k) order[k] = k;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return keys[a] < keys[b]; });
  std::vector<int> ri(keys.size()), ci(keys.size());
  std::vector<double> v(keys.size());
  for (size_t k = 0; k < order.size(); ++k) {
    uint64_t key = keys[order[k]];
    ci[k] = (int)(key / (uint64_t)m);
    ri[k] = (int)(key % (uint64_t)m);
    v[k] = vals[order[k]];
  }
  lp_problem_t *p = alloc_problem(m, n, (long)nnz);
  if (!p) return nullptr;
  coo_cols_to_csr(p, ri, ci, v);
  feasible_bounds(p, rng);
  return p;
}

lp_problem_t *pdlp_generate_powerlaw_lp(int m, int n, long long nnz_target, double zipf_s,
                                        int max_degree, unsigned long long seed) {
  if (m <= 0 || n <= 0 || nnz_target <= 0 || max_degree <= 0 || zipf_s <= 0) return nullptr;
  if (max_degree > m) max_degree = m;
  // rank weights r^-s
  std::vector<double> w(n);
  for (int r = 1; r <= n; ++r) w[r - 1] = det_exp(-zipf_s * det_log((double)r));
  auto degree_sum = [&](double C, std::vector<int> *out) {
    long long s = 0;
    for (int r = 0; r < n; ++r) {
      double d = floor(C * w[r] + 0.5);
      long long di = d < 1.0 ? 1 : (d > max_degree ? max_degree : (long long)d);
      s += di;
      if (out) (*out)[r] = (int)di;
    }
    return s;
  };
  double lo = 0.0, hi = 1.0;
  while (degree_sum(hi, nullptr) < nnz_target && hi < 1e18) hi *= 2.0;
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (degree_sum(mid, nullptr) < nnz_target) lo = mid;
    else hi = mid;
  }
  std::vector<int> deg(n);
  long long total = degree_sum(hi, &deg);
  if (total > 2000000000LL) return nullptr;
  Rng rng(seed);
  // random column for each rank (Fisher-Yates)
  std::vector<int> col_of_rank(n);
  for (int j = 0; j < n; ++j) col_of_rank[j] = j;
  for (int j = n - 1; j > 0; --j) std::swap(col_of_rank[j], col_of_rank[rng.below((uint64_t)j + 1)]);
  std::vector<int> col_deg(n);
  for (int r = 0; r < n; ++r) col_deg[col_of_rank[r]] = deg[r];
  std::vector<int> ri, ci;
  std::vector<double> v;
  ri.reserve((size_t)total);
  ci.reserve((size_t)total);
  v.reserve((size_t)total);
  // distinct rows per column: stamp[r] == j marks row r as taken by column j
  std::vector<int> stamp((size_t)m, -1);
  for (int j = 0; j < n; ++j) {
    int d = col_deg[j], got = 0;
    while (got < d) {
      int r = (int)rng.below((uint64_t)m);
      if (stamp[r] == j) continue;
      stamp[r] = j;
      ++got;
      ri.push_back(r);
      ci.push_back(j);
      double u = rng.uniform();
      double val;
      if (u < 0.05) val = (rng.next() & 1) ? 1.0 : -1.0;
      else val = rng.normal();
      v.push_back(val);
    }
  }
  lp_problem_t *p = alloc_problem(m, n, (long)total);
  if (!p) return nullptr;
  coo_cols_to_csr(p, ri, ci, v);
  feasible_bounds(p, rng);
  return p;
}

lp_problem_t *pdlp_generate_transport_lp(int sources, int sinks, unsigned long long seed) {
  if (sources <= 0 || sinks <= 0) return nullptr;
  long long n = (long long)sources * sinks;
  if (n * 2 > 2000000000LL) return nullptr;
  const int m = sources + sinks;
  lp_problem_t *p = alloc_problem(m, (int)n, (long)(2 * n));
  if (!p) return nullptr;
  Rng rng(seed);
  std::vector<double> supply(sources), demand(sinks);
  double ssum = 0.0, dsum = 0.0;
  for (int i = 0; i < sources; ++i) ssum += (supply[i] = 1.0 + 99.0 * rng.uniform());
  for (int j = 0; j < sinks; ++j) dsum += (demand[j] = 1.0 + 99.0 * rng.uniform());
  for (int j = 0; j < sinks; ++j) demand[j] *= ssum / dsum;
  int *rp = p->constraint_matrix_row_pointers;
  int *cj = p->constraint_matrix_col_indices;
  double *av = p->constraint_matrix_values;
  long k = 0;
  // source rows: arcs i*sinks + j, j ascending
  for (int i = 0; i < sources; ++i) {
    rp[i] = (int)k;
    for (int j = 0; j < sinks; ++j) {
      cj[k] = (int)((long long)i * sinks + j);
      av[k++] = 1.0;
    }
  }
  // sink rows: arcs i*sinks + j, i ascending
  for (int j = 0; j < sinks; ++j) {
    rp[sources + j] = (int)k;
    for (int i = 0; i < sources; ++i) {
      cj[k] = (int)((long long)i * sinks + j);
      av[k++] = 1.0;
    }
  }
  rp[m] = (int)k;
  for (int i = 0; i < sources; ++i)
    p->constraint_lower_bound[i] = p->constraint_upper_bound[i] = supply[i];
  for (int j = 0; j < sinks; ++j)
    p->constraint_lower_bound[sources + j] = p->constraint_upper_bound[sources + j] = demand[j];
  for (long long a = 0; a < n; ++a) {
    p->objective_vector[a] = rng.uniform();
    p->variable_lower_bound[a] = 0.0;
    p->variable_upper_bound[a] = INFINITY;
  }
  p->objective_constant = 0.0;
  return p;
}

}  // extern "C"
