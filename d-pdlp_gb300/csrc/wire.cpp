// wire.cpp -- binary problem format for request payloads and stored instances.
//
// The byte layout of the reference's serialize_lp_problem_to_ptr /
// deserialize_lp_problem_from_ptr (src/distribution_utils.cu:279-405), so a
// payload written by either side reads on the other:
//   int32 n, int32 m, int32 nnz, float64 objective constant,
//   float64 c[n], lv[n], uv[n], lc[m], uc[m],
//   int32 row_ptr[m+1], int32 col[nnz], float64 val[nnz],
//   int32 has_primal_start, int32 has_dual_start,
//   float64 primal_start[n] (if any), float64 dual_start[m] (if any)
// in the host's byte order, packed (no padding).  Reading checks every count
// against the buffer length and the CSR against the sizes -- the reference
// trusts the payload -- and builds the problem through create_lp_problem.
#include <stdint.h>
#include <string.h>

#include "cupdlpx.h"
#include "pdlp_gb300.h"

namespace {

struct Reader {
  const unsigned char *p;
  long long left;
  template <class V>
  bool get(V &v) {
    if (left < (long long)sizeof(V)) return false;
    memcpy(&v, p, sizeof(V));
    p += sizeof(V);
    left -= sizeof(V);
    return true;
  }
  const unsigned char *take(long long bytes) {
    if (bytes < 0 || left < bytes) return nullptr;
    const unsigned char *q = p;
    p += bytes;
    left -= bytes;
    return q;
  }
};

}  // namespace

extern "C" {

long long pdlp_problem_wire_size(const lp_problem_t *lp) {
  if (!lp) return -1;
  const long long n = lp->num_variables, m = lp->num_constraints,
                  nnz = lp->constraint_matrix_num_nonzeros;
  long long b = 3 * 4 + 8 + 8 * (3 * n + 2 * m) + 4 * (m + 1) + 12 * nnz + 2 * 4;
  if (lp->primal_start) b += 8 * n;
  if (lp->dual_start) b += 8 * m;
  return b;
}

long long pdlp_problem_serialize(const lp_problem_t *lp, void *buf, long long capacity) {
  const long long size = pdlp_problem_wire_size(lp);
  if (size < 0 || !buf || capacity < size) return -1;
  unsigned char *o = (unsigned char *)buf;
  auto put = [&](const void *src, long long bytes) {
    if (bytes > 0) memcpy(o, src, (size_t)bytes);
    o += bytes;
  };
  const int n = lp->num_variables, m = lp->num_constraints,
            nnz = lp->constraint_matrix_num_nonzeros;
  put(&n, 4);
  put(&m, 4);
  put(&nnz, 4);
  put(&lp->objective_constant, 8);
  put(lp->objective_vector, 8LL * n);
  put(lp->variable_lower_bound, 8LL * n);
  put(lp->variable_upper_bound, 8LL * n);
  put(lp->constraint_lower_bound, 8LL * m);
  put(lp->constraint_upper_bound, 8LL * m);
  put(lp->constraint_matrix_row_pointers, 4LL * ((long long)m + 1));
  put(lp->constraint_matrix_col_indices, 4LL * nnz);
  put(lp->constraint_matrix_values, 8LL * nnz);
  const int hp = lp->primal_start != nullptr, hd = lp->dual_start != nullptr;
  put(&hp, 4);
  put(&hd, 4);
  if (hp) put(lp->primal_start, 8LL * n);
  if (hd) put(lp->dual_start, 8LL * m);
  return size;
}

lp_problem_t *pdlp_problem_deserialize(const void *buf, long long length) {
  if (!buf || length < 0) return nullptr;
  Reader r{(const unsigned char *)buf, length};
  int n = 0, m = 0, nnz = 0;
  double c0 = 0.0;
  if (!r.get(n) || !r.get(m) || !r.get(nnz) || !r.get(c0)) return nullptr;
  if (n < 0 || m < 0 || nnz < 0) return nullptr;
  const unsigned char *c = r.take(8LL * n), *lv = r.take(8LL * n), *uv = r.take(8LL * n);
  const unsigned char *lc = r.take(8LL * m), *uc = r.take(8LL * m);
  const unsigned char *rp = r.take(4LL * ((long long)m + 1)), *ci = r.take(4LL * nnz);
  const unsigned char *vx = r.take(8LL * nnz);
  int hp = 0, hd = 0;
  if (!c || !lv || !uv || !lc || !uc || !rp || !ci || !vx || !r.get(hp) || !r.get(hd))
    return nullptr;
  const unsigned char *ps = hp ? r.take(8LL * n) : nullptr;
  const unsigned char *ds = hd ? r.take(8LL * m) : nullptr;
  if ((hp && !ps) || (hd && !ds)) return nullptr;
  // copies with the alignment create_lp_problem's arrays need
  auto dvec = [](const unsigned char *src, long long k) {
    double *v = (double *)malloc(sizeof(double) * (size_t)(k ? k : 1));
    if (v && k) memcpy(v, src, sizeof(double) * (size_t)k);
    return v;
  };
  auto ivec = [](const unsigned char *src, long long k) {
    int *v = (int *)malloc(sizeof(int) * (size_t)(k ? k : 1));
    if (v && k) memcpy(v, src, sizeof(int) * (size_t)k);
    return v;
  };
  double *cv = dvec(c, n), *lvv = dvec(lv, n), *uvv = dvec(uv, n), *lcv = dvec(lc, m),
         *ucv = dvec(uc, m), *vv = dvec(vx, nnz), *psv = hp ? dvec(ps, n) : nullptr,
         *dsv = hd ? dvec(ds, m) : nullptr;
  int *rpv = ivec(rp, (long long)m + 1), *civ = ivec(ci, nnz);
  lp_problem_t *lp = nullptr;
  bool ok = cv && lvv && uvv && lcv && ucv && vv && rpv && civ && (!hp || psv) && (!hd || dsv);
  // the CSR must describe m rows and nnz entries in [0, n)
  if (ok) ok = rpv[0] == 0 && rpv[m] == nnz;
  for (int i = 0; ok && i < m; ++i) ok = rpv[i] <= rpv[i + 1];
  for (int k = 0; ok && k < nnz; ++k) ok = civ[k] >= 0 && civ[k] < n;
  if (ok) {
    matrix_desc_t A{};
    A.m = m;
    A.n = n;
    A.fmt = matrix_csr;
    A.zero_tolerance = 0.0;
    A.data.csr.nnz = nnz;
    A.data.csr.row_ptr = rpv;
    A.data.csr.col_ind = civ;
    A.data.csr.vals = vv;
    lp = create_lp_problem(cv, &A, lcv, ucv, lvv, uvv, &c0);
    if (lp && (hp || hd)) set_start_values(lp, psv, dsv);
  }
  free(cv); free(lvv); free(uvv); free(lcv); free(ucv); free(vv);
  free(psv); free(dsv); free(rpv); free(civ);
  return lp;
}

long long pdlp_server_submit_bytes(pdlp_server_t *s, const void *buf, long long length) {
  lp_problem_t *lp = pdlp_problem_deserialize(buf, length);
  if (!lp) return -1;
  long long id = pdlp_server_submit(s, lp);
  lp_problem_free(lp);
  return id;
}

}  // extern "C"
