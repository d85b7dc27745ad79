// C-ABI entry points: context, integral tables, determinant set, sigma.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "qpgpu_internal.cuh"

int qpgpu_fail(qpgpu_ctx* c, int code, const std::string& msg) {
  if (c) c->last_error = msg;
  return code;
}

namespace {

inline unsigned gsz(int64_t n, int tpb = 256) {
  int64_t g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > 65535LL * 64) g = 65535LL * 64;
  return (unsigned)g;
}

// mo_bielec_integral_jj / _exchange / _anti, mo_bi_integrals.irp.f:1344-1369
__global__ void k_tables2(DevTables t, double* jj, double* kk, double* ja) {
  const int n = t.n;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < (int64_t)n * n; x += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(x % n) + 1, j = (int)(x / n) + 1;
    const double a = get_int(t, i, j, i, j), b = get_int(t, i, j, j, i);
    jj[x] = a;
    kk[x] = b;
    ja[x] = __dsub_rn(a, b);
  }
}

// big_array_coulomb/exchange_integrals(j,i,k) = <ij|kj>, <ij|jk>, integrals_3_index.irp.f:1-22
__global__ void k_tables3(DevTables t, double* bc, double* bx) {
  const int64_t n = t.n;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n * n * n; x += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(x % n) + 1, i = (int)((x / n) % n) + 1, k = (int)(x / (n * n)) + 1;
    bc[x] = get_int(t, i, j, k, j);
    bx[x] = get_int(t, i, j, j, k);
  }
}

// fock_operator_closed_shell_ref_bitmask, mono_excitations.irp.f:22-95:
// F(i,j) = sum_{k in docc, ascending} (2 <ik|jk> - <ik|kj>) + h(i,j)
__global__ void k_fock(DevTables t, double* fock) {
  const int n = t.n;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < (int64_t)n * n; x += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(x % n) + 1, j = (int)(x / n) + 1;
    double accu = 0.0;
    for (int w = 0; w < t.nint; ++w)
      for (u64 b = t.ref_cs[w]; b; b &= b - 1) {
        const int k = ctz64(b) + 1 + 64 * w;
        accu = __dadd_rn(accu, __dsub_rn(2.0 * get_int(t, i, k, j, k), get_int(t, i, k, k, j)));
      }
    fock[x] = __dadd_rn(accu, tab2(t.h, n, i, j));
  }
}

// ref_bitmask_energy, ref_bitmask.irp.f:1-56 (reference occupations 1..N_a / 1..N_b)
__global__ void k_eref(DevTables t, double* out) {
  if (blockIdx.x || threadIdx.x) return;
  const int n = t.n, na = t.na, nb = t.nb;
  double e = 0.0;
  for (int i = 1; i <= nb; ++i) e = __dadd_rn(e, __dadd_rn(tab2(t.h, n, i, i), tab2(t.h, n, i, i)));
  for (int i = nb + 1; i <= na; ++i) e = __dadd_rn(e, tab2(t.h, n, i, i));
  for (int j = 1; j <= na; ++j)
    for (int i = j + 1; i <= na; ++i) e = __dadd_rn(e, tab2(t.ja, n, i, j));
  for (int j = 1; j <= nb; ++j) {
    for (int i = j + 1; i <= nb; ++i) e = __dadd_rn(e, tab2(t.ja, n, i, j));
    for (int i = 1; i <= na; ++i) e = __dadd_rn(e, tab2(t.jj, n, i, j));
  }
  *out = e;
}

// connected-pair export (debug): class, phase and excitation of stored pair e
// (row k) into record o, with the get_mono/double_excitation_spin routines
// (slater_rules.irp.f:2783-2987)
struct PairOut {
  int32_t* I;
  int32_t* J;
  int8_t* cls;
  int8_t* phase;
  int16_t* exc;
  double* hij;
};

template <int NINT>
__device__ void export_pair(const DevTables& t, const u64* alpha, const u64* beta, const int* rows, const int* cols,
                            const int* order, const int* colidx, const double* val, int k, int64_t e, int64_t o,
                            const PairOut& out) {
  const int jp = colidx[e];
  u64 di[2 * NINT], dj[2 * NINT];
  for (int w = 0; w < NINT; ++w) {
    di[w] = alpha[(int64_t)rows[k] * NINT + w];
    di[NINT + w] = beta[(int64_t)cols[k] * NINT + w];
    dj[w] = alpha[(int64_t)rows[jp] * NINT + w];
    dj[NINT + w] = beta[(int64_t)cols[jp] * NINT + w];
  }
  int da = 0, db = 0;
  for (int w = 0; w < NINT; ++w) {
    da += popc64(di[w] ^ dj[w]);
    db += popc64(di[NINT + w] ^ dj[NINT + w]);
  }
  int c, neg = 0, x4[4] = {0, 0, 0, 0};
  double s2;
  if (db == 0) {
    c = (da == 2) ? 1 : 3;
    if (c == 1) h_mono_spin<NINT>(t, di, dj, 1, x4, &neg);
    else h_double_spin<NINT>(t, di, dj, x4, &neg);
  } else if (da == 0) {
    c = (db == 2) ? 2 : 4;
    if (c == 2) h_mono_spin<NINT>(t, di, dj, 2, x4, &neg);
    else h_double_spin<NINT>(t, di + NINT, dj + NINT, x4, &neg);
  } else {
    c = 5;
    h_double_ab<NINT>(t, di, dj, &s2, x4, &neg);
  }
  out.I[o] = order[k];
  out.J[o] = order[jp];
  out.cls[o] = (int8_t)c;
  out.phase[o] = neg ? -1 : 1;
  for (int q = 0; q < 4; ++q) out.exc[4 * o + q] = (int16_t)x4[q];
  out.hij[o] = val[e];
}

// pairs of selected rows: block b exports the pairs of bilinear row rsel[b]
// into records starting at obeg[b]
template <int NINT>
__global__ void k_export_rows(DevTables t, const u64* alpha, const u64* beta, const int* rows, const int* cols,
                              const int* order, const int64_t* rowptr, const int* colidx, const double* val,
                              const int* rsel, const int64_t* obeg, int nsel, PairOut out) {
  for (int b = blockIdx.x; b < nsel; b += gridDim.x) {
    const int k = rsel[b];
    const int64_t rb = rowptr[k], re = rowptr[k + 1];
    for (int64_t e = rb + threadIdx.x; e < re; e += blockDim.x)
      export_pair<NINT>(t, alpha, beta, rows, cols, order, colidx, val, k, e, obeg[b] + (e - rb), out);
  }
}

template <int NINT>
__global__ void k_export_pairs(DevTables t, const u64* alpha, const u64* beta, const int* rows, const int* cols,
                               const int* order, const int64_t* rowptr, const int* colidx, const double* val,
                               int64_t N, int64_t P, int32_t* I, int32_t* J, int8_t* cls, int8_t* phase,
                               int16_t* exc, double* hij) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = N;  // last k with rowptr[k] <= e
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (rowptr[mid] <= e) lo = mid; else hi = mid;
    }
    export_pair<NINT>(t, alpha, beta, rows, cols, order, colidx, val, (int)lo, e, e,
                      PairOut{I, J, cls, phase, exc, hij});
  }
}

int check_ctx(qpgpu_ctx* c, bool need_ints, bool need_dets) {
  if (!c) return QPGPU_ERR_ARG;
  if (need_ints && !c->have_ints) return qpgpu_fail(c, QPGPU_ERR_STATE, "integrals not set");
  if (need_dets && !c->have_pairs) return qpgpu_fail(c, QPGPU_ERR_STATE, "determinants not set");
  return 0;
}

void free_ints(qpgpu_ctx* c) {
  double** ps[] = {&c->d_eri, &c->d_h, &c->d_jj, &c->d_kk, &c->d_ja, &c->d_bc, &c->d_bx, &c->d_fock, &c->d_eref};
  for (auto p : ps) {
    dev_free(*p);
    *p = nullptr;
  }
  c->have_ints = false;
}

int ensure_work(qpgpu_ctx* c, size_t bytes) {
  if (c->work_bytes >= bytes) return 0;
  dev_free(c->d_work);
  c->d_work = nullptr;
  c->work_bytes = 0;
  QP_CUDA(c, cudaMalloc((void**)&c->d_work, bytes));
  c->work_bytes = bytes;
  return 0;
}

}  // namespace

void qp_report_marks(qpgpu_ctx* c) {
  if (!c->profile || c->marks.size() < 2) return;
  cudaEventSynchronize(c->marks.back().second);
  for (size_t i = 1; i < c->marks.size(); ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->marks[i - 1].second, c->marks[i].second);
    fprintf(stderr, "[qpgpu] %-22s %10.3f ms\n", c->marks[i].first.c_str(), ms);
  }
  for (auto& m : c->marks) cudaEventDestroy(m.second);
  c->marks.clear();
}

int qp_numeric_flag(qpgpu_ctx* c, cudaStream_t st, int** flag) {
  if (!c->d_flag) QP_CUDA(c, cudaMalloc((void**)&c->d_flag, 64));
  QP_CUDA(c, cudaMemsetAsync(c->d_flag, 0, sizeof(int), st));
  *flag = c->d_flag;
  return 0;
}

namespace {

struct Lock {
  std::mutex& m;
  explicit Lock(std::mutex& mm) : m(mm) { m.lock(); }
  ~Lock() { m.unlock(); }
};

}  // namespace

extern "C" {

int qpgpu_create(int n_mo, int n_alpha, int n_beta, int n_int, qpgpu_ctx** out) {
  if (!out) return QPGPU_ERR_ARG;
  *out = nullptr;
  if (n_mo < 1 || n_mo > QPGPU_MAX_MO || n_int != (n_mo - 1) / 64 + 1 || n_alpha < n_beta || n_beta < 0 ||
      n_alpha > n_mo)
    return QPGPU_ERR_ARG;
  qpgpu_ctx* c = new qpgpu_ctx();
  c->n_mo = n_mo;
  c->na = n_alpha;
  c->nb = n_beta;
  c->nint = n_int;
  {
    const char* pe = getenv("QPGPU_PROFILE");
    c->profile = pe && pe[0] == '1';
  }
  if (cudaGetDevice(&c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return QPGPU_ERR_CUDA;
  }
  if (cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || c->n_sm < 1) {
    cudaGetLastError();
    cudaStreamDestroy(c->stream);
    delete c;
    return QPGPU_ERR_CUDA;
  }
  *out = c;
  return QPGPU_OK;
}

int qpgpu_destroy(qpgpu_ctx* c) {
  if (!c) return QPGPU_ERR_ARG;
  {
    Lock l(c->mu);
    cudaStreamSynchronize(c->stream);
    c->items.free_all();
    qp_free_dressing(c);
    qp_free_pairs(c);
    qp_free_dets(c);
    free_ints(c);
    c->mlp.free_all();
    dev_free(c->d_work);
    dev_free(c->d_stage);
    dev_free(c->d_ffu);
    dev_free(c->d_direct_ut);
    dev_free(c->d_flag);
    dev_free(c->d_tc_scratch);
    cudaStreamDestroy(c->stream);
  }
  delete c;
  return QPGPU_OK;
}

const char* qpgpu_last_error(qpgpu_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int qpgpu_get_info(qpgpu_ctx* c, qpgpu_info* info) {
  if (!c || !info) return QPGPU_ERR_ARG;
  Lock l(c->mu);
  info->n_det = c->N;
  info->n_alpha_unique = c->Ua;
  info->n_beta_unique = c->Ub;
  info->n_pairs = c->P;
  info->n_s2_pairs = c->P_s2;
  info->setup_ms = c->setup_ms;
  info->ref_energy = c->tab.e_ref;
  const int64_t n = c->n_mo, N = c->N, P = c->P;
  int64_t b = 0;
  if (c->have_ints) b += 8 * (n * (n + 1) / 2) * (n * (n + 1) / 2 + 1) / 2 + 8 * (6 * n * n + 2 * n * n * n);
  if (c->have_dets) b += N * (32 * c->nint + 4 * 8) + 8 * (int64_t)(c->Ua + c->Ub) * c->nint;
  if (c->have_pairs && !c->direct) b += P * 16 + c->P_s2 * 8 + N * 28;
  if (c->have_pairs && c->direct) b += N * 24;
  for (int k = 0; k < KT_N; ++k) b += c->kslots[k] * (int64_t)sizeof(KeySlot) + c->kmem_n[k] * 4;
  if (c->have_dets) b += c->Ua + c->Ub;
  b += (int64_t)c->work_bytes;
  info->device_bytes = b;
  info->n_split_rows = c->items.n_multi;
  info->direct_sigma = c->direct ? 1 : 0;
  info->n_keyed_lines = c->n_keyed_lines;
  return QPGPU_OK;
}

int qpgpu_set_sigma_mode(qpgpu_ctx* c, int mode) {
  if (!c) return QPGPU_ERR_ARG;
  if (mode != QPGPU_SIGMA_AUTO && mode != QPGPU_SIGMA_STORED && mode != QPGPU_SIGMA_DIRECT)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "sigma mode must be QPGPU_SIGMA_AUTO, _STORED or _DIRECT");
  Lock l(c->mu);
  c->sigma_mode = mode;
  return QPGPU_OK;
}

int qpgpu_set_line_keys(qpgpu_ctx* c, int64_t min_single, int64_t min_double, int hash_bits) {
  if (!c) return QPGPU_ERR_ARG;
  if (min_single < -1 || min_double < -1 || hash_bits < 1 || hash_bits > 64)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "line keys: thresholds must be >= -1 and hash_bits in 1..64");
  Lock l(c->mu);
  c->key_min_single = min_single;
  c->key_min_double = min_double;
  c->key_hash_bits = hash_bits;
  return QPGPU_OK;
}

int qpgpu_set_integrals(qpgpu_ctx* c, const double* h, const double* eri) {
  if (!c || !h || !eri) return QPGPU_ERR_ARG;
  Lock l(c->mu);
  const int n = c->n_mo;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (h[i + (size_t)j * n] != h[j + (size_t)i * n])
        return qpgpu_fail(c, QPGPU_ERR_ARG, "h_pq must be symmetric");
  c->items.free_all();
  qp_free_dressing(c);
  qp_free_pairs(c);
  qp_free_dets(c);
  free_ints(c);
  const int64_t p2 = (int64_t)n * (n + 1) / 2;
  const int64_t npk = p2 * (p2 + 1) / 2;
  cudaStream_t st = c->stream;
  if (dev_alloc(&c->d_eri, npk) != cudaSuccess || dev_alloc(&c->d_h, (size_t)n * n) != cudaSuccess ||
      dev_alloc(&c->d_jj, (size_t)n * n) != cudaSuccess || dev_alloc(&c->d_kk, (size_t)n * n) != cudaSuccess ||
      dev_alloc(&c->d_ja, (size_t)n * n) != cudaSuccess || dev_alloc(&c->d_fock, (size_t)n * n) != cudaSuccess ||
      dev_alloc(&c->d_bc, (size_t)n * n * n) != cudaSuccess || dev_alloc(&c->d_bx, (size_t)n * n * n) != cudaSuccess ||
      dev_alloc(&c->d_eref, 1) != cudaSuccess) {
    cudaGetLastError();
    free_ints(c);
    return qpgpu_fail(c, QPGPU_ERR_NOMEM, "integral tables do not fit on the device");
  }
  QP_CUDA(c, cudaMemcpyAsync(c->d_eri, eri, npk * sizeof(double), cudaMemcpyHostToDevice, st));
  QP_CUDA(c, cudaMemcpyAsync(c->d_h, h, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice, st));
  DevTables& t = c->tab;
  t = DevTables{};
  t.n = n;
  t.nint = c->nint;
  t.na = c->na;
  t.nb = c->nb;
  t.eri = c->d_eri;
  t.h = c->d_h;
  t.jj = c->d_jj;
  t.ja = c->d_ja;
  t.bc = c->d_bc;
  t.bx = c->d_bx;
  t.fock = c->d_fock;
  // ref_bitmask = HF_bitmask (bitmasks.irp.f:71-95); closed-shell reference
  // keeps the N_beta lowest orbitals in both spins (mono_excitations.irp.f:2-19)
  for (int i = 0; i < c->na; ++i) t.ref[i >> 6] |= 1ull << (i & 63);
  for (int i = 0; i < c->nb; ++i) t.ref[c->nint + (i >> 6)] |= 1ull << (i & 63);
  for (int i = 0; i < c->nb; ++i) {
    t.ref_cs[i >> 6] |= 1ull << (i & 63);
    t.ref_cs[c->nint + (i >> 6)] |= 1ull << (i & 63);
  }
  k_tables2<<<gsz((int64_t)n * n), 256, 0, st>>>(t, c->d_jj, c->d_kk, c->d_ja);
  k_tables3<<<gsz((int64_t)n * n * n), 256, 0, st>>>(t, c->d_bc, c->d_bx);
  k_fock<<<gsz((int64_t)n * n), 256, 0, st>>>(t, c->d_fock);
  k_eref<<<1, 32, 0, st>>>(t, c->d_eref);
  QP_CUDA(c, cudaGetLastError());
  QP_CUDA(c, cudaMemcpyAsync(&t.e_ref, c->d_eref, sizeof(double), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  c->have_ints = true;
  return QPGPU_OK;
}

int qpgpu_set_dets(qpgpu_ctx* c, const uint64_t* psi_det, int64_t n_det) {
  int rc = check_ctx(c, true, false);
  if (rc) return rc;
  if (!psi_det || n_det < 1 || n_det >= ((int64_t)1 << 31) - 1) return qpgpu_fail(c, QPGPU_ERR_ARG, "bad n_det");
  Lock l(c->mu);
  // every determinant must hold N_alpha / N_beta electrons within n_mo orbitals
  const int nint = c->nint;
  for (int64_t k = 0; k < n_det; ++k) {
    for (int s = 0; s < 2; ++s) {
      int cnt = 0;
      for (int w = 0; w < nint; ++w) {
        const uint64_t x = psi_det[(k * 2 + s) * nint + w];
        cnt += __builtin_popcountll(x);
        const int hi = c->n_mo - 64 * w;
        if (hi < 64 && (x >> (hi > 0 ? hi : 0)) != 0)
          return qpgpu_fail(c, QPGPU_ERR_ARG, "determinant " + std::to_string(k) + " uses orbitals > n_mo");
      }
      if (cnt != (s == 0 ? c->na : c->nb))
        return qpgpu_fail(c, QPGPU_ERR_ARG, "determinant " + std::to_string(k) + " has a wrong electron count");
    }
  }
  c->items.free_all();
  qp_free_dressing(c);
  qp_free_pairs(c);
  qp_free_dets(c);
  cudaStream_t st = c->stream;
  cudaEvent_t e0, e1;
  QP_CUDA(c, cudaEventCreate(&e0));
  QP_CUDA(c, cudaEventCreate(&e1));
  QP_CUDA(c, dev_alloc(&c->d_dets, (size_t)n_det * 2 * nint));
  QP_CUDA(c, cudaMemcpyAsync(c->d_dets, psi_det, (size_t)n_det * 2 * nint * 8, cudaMemcpyHostToDevice, st));
  QP_CUDA(c, cudaEventRecord(e0, st));
  qp_mark(c, "start");
  c->N = n_det;
  rc = qp_build_index(c);
  if (rc == 0) {
    c->have_dets = true;
    rc = qp_build_pairs(c);
  }
  if (rc == 0 && !c->direct) rc = qp_build_sigma_items(c, &c->items);
  if (rc == 0) rc = qp_det_features(c);
  qp_mark(c, "sigma work items");
  qp_report_marks(c);
  QP_CUDA(c, cudaEventRecord(e1, st));
  QP_CUDA(c, cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) {
    c->items.free_all();
    qp_free_pairs(c);
    qp_free_dets(c);
    return rc;
  }
  c->setup_ms = ms;
  c->have_pairs = true;
  return QPGPU_OK;
}

int qpgpu_sigma_bilinear(qpgpu_ctx* c, double* v_t, double* s_t, const double* u_t, const float* u_t32, int n_st,
                         int precision, void* stream) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  if (!v_t || !s_t || !u_t || n_st < 1 || n_st > 8 ||
      (precision != QPGPU_FP64 && precision != QPGPU_FP32 && precision != QPGPU_FF))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "bad sigma arguments (n_st must be 1..8)");
  if (((uintptr_t)u_t & 15) || (u_t32 && ((uintptr_t)u_t32 & 15)))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "u_t and u_t32 must be 16-byte aligned");
  Lock l(c->mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  if (precision == QPGPU_FF) return qp_sigma_ff(c, &c->items, v_t, s_t, u_t, n_st, st, 0, (int)c->N, 0, 1);
  return qp_sigma_launch(c, &c->items, v_t, s_t, u_t, u_t32, n_st, precision, st, 0, (int)c->N, 0, 1);
}

}  // extern "C"

namespace {
// qpgpu_h_s2_u0_device with an optional device flag that the input conversion
// sets when u0 holds a NaN or an infinity (called with the context locked)
int h_s2_u0_dev(qpgpu_ctx* c, double* v0, double* s0, const double* u0, int n_st, int64_t ld, int precision,
                cudaStream_t st, int* bad, bool dressed = false) {
  const int64_t N = c->N;
  int rc = 0;
  const int nb = n_st < 8 ? n_st : 8;
  rc = ensure_work(c, (size_t)N * nb * (3 * sizeof(double) + sizeof(float)) + 1024);
  if (rc) return rc;
  double* ut = c->d_work;
  double* vt = ut + (size_t)N * nb;
  double* stt = vt + (size_t)N * nb;
  float* ut32 = (float*)(stt + (size_t)N * nb);
  for (int s0i = 0; s0i < n_st; s0i += 8) {
    const int m = (n_st - s0i) < 8 ? (n_st - s0i) : 8;
    qp_to_bilinear(u0 + (int64_t)s0i * ld, ld, c->d_order, ut, precision == QPGPU_FP32 ? ut32 : nullptr, m, N, st,
                   bad);
    rc = qp_sigma_launch(c, &c->items, vt, stt, ut, ut32, m, precision, st, 0, (int)N, 0, 1);
    if (!rc && dressed) rc = qp_dress(c, vt, stt, ut, m, st);
    if (rc) return rc;
    qp_from_bilinear(vt, ld, c->d_order, v0 + (int64_t)s0i * ld, m, N, st);
    qp_from_bilinear(stt, ld, c->d_order, s0 + (int64_t)s0i * ld, m, N, st);
  }
  QP_CUDA(c, cudaGetLastError());
  return QPGPU_OK;
}
}  // namespace

extern "C" {

int qpgpu_h_s2_u0_device(qpgpu_ctx* c, double* v0, double* s0, const double* u0, int n_st, int64_t ld,
                         int precision, void* stream) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  if (!v0 || !s0 || !u0 || n_st < 1 || ld < c->N || (precision != QPGPU_FP64 && precision != QPGPU_FP32))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "bad h_s2_u0 arguments");
  Lock l(c->mu);
  return h_s2_u0_dev(c, v0, s0, u0, n_st, ld, precision, stream ? (cudaStream_t)stream : c->stream, nullptr);
}

namespace {
int h_s2_u0_host(qpgpu_ctx* c, double* v0, double* s0, const double* u0, int n_st, int64_t ld, bool dressed) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  if (!v0 || !s0 || !u0 || n_st < 1 || ld < c->N) return qpgpu_fail(c, QPGPU_ERR_ARG, "bad h_s2_u0 arguments");
  const int64_t N = c->N;
  const size_t cols = (size_t)N * n_st;
  Lock l(c->mu);
  if (c->stage_bytes < 3 * cols * sizeof(double)) {
    dev_free(c->d_stage);
    c->d_stage = nullptr;
    c->stage_bytes = 0;
    QP_CUDA(c, cudaMalloc((void**)&c->d_stage, 3 * cols * sizeof(double)));
    c->stage_bytes = 3 * cols * sizeof(double);
  }
  double *du = c->d_stage, *dv = du + cols, *ds = du + 2 * cols;
  cudaStream_t st = c->stream;
  int* bad = nullptr;
  rc = qp_numeric_flag(c, st, &bad);
  if (rc) return rc;
  int hbad = 0;
  if (cudaMemcpy2DAsync(du, N * sizeof(double), u0, ld * sizeof(double), N * sizeof(double), n_st,
                        cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = qpgpu_fail(c, QPGPU_ERR_CUDA, "copy of u_0 failed");
  if (!rc && dressed && !c->dress.on) rc = qpgpu_fail(c, QPGPU_ERR_STATE, "no dressing set");
  if (!rc) rc = h_s2_u0_dev(c, dv, ds, du, n_st, N, QPGPU_FP64, st, bad, dressed);
  if (!rc && (cudaMemcpy2DAsync(v0, ld * sizeof(double), dv, N * sizeof(double), N * sizeof(double), n_st,
                                cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpy2DAsync(s0, ld * sizeof(double), ds, N * sizeof(double), N * sizeof(double), n_st,
                                cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess))
    rc = qpgpu_fail(c, QPGPU_ERR_CUDA, "copy of v_0/s_0 failed");
  cudaError_t e = cudaStreamSynchronize(st);
  if (!rc && e != cudaSuccess) rc = qpgpu_fail(c, QPGPU_ERR_CUDA, cudaGetErrorString(e));
  if (!rc && hbad) rc = qpgpu_fail(c, QPGPU_ERR_NUMERIC, "u_0 holds a NaN or an infinity");
  return rc;
}

}  // namespace

int qpgpu_h_s2_u0(qpgpu_ctx* c, double* v0, double* s0, const double* u0, int n_st, int64_t ld) {
  return h_s2_u0_host(c, v0, s0, u0, n_st, ld, false);
}

int qpgpu_h_s2_u0_dressed(qpgpu_ctx* c, double* v0, double* s0, const double* u0, int n_st, int64_t ld) {
  return h_s2_u0_host(c, v0, s0, u0, n_st, ld, true);
}

namespace {
constexpr int DOT_CTA = 256;
inline int dot_grid(const qpgpu_ctx* c) { return 2 * c->n_sm; }  // two CTAs per SM
// per-CTA partial sums of u.u and u.v for each column (fixed summation order)
__global__ void k_col_dots(const double* u, const double* v, int64_t N, int n_st, double* partial) {
  __shared__ double red[2][DOT_CTA / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < n_st; ++i) {
    const double* ui = u + (int64_t)i * N;
    const double* vi = v + (int64_t)i * N;
    double uu = 0.0, uv = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)DOT_CTA + threadIdx.x; r < N; r += (int64_t)gridDim.x * DOT_CTA) {
      uu = fma(ui[r], ui[r], uu);
      uv = fma(ui[r], vi[r], uv);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      uu += __shfl_xor_sync(0xffffffffu, uu, o);
      uv += __shfl_xor_sync(0xffffffffu, uv, o);
    }
    if (lane == 0) {
      red[0][w] = uu;
      red[1][w] = uv;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
      double t = 0.0;
      for (int q = 0; q < DOT_CTA / 32; ++q) t += red[threadIdx.x][q];
      partial[((int64_t)blockIdx.x * n_st + i) * 2 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}
}  // namespace

int qpgpu_u0_h_u0(qpgpu_ctx* c, double* e_0, const double* u0, int n_st, int64_t ld) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  if (!e_0 || !u0 || n_st < 1 || ld < c->N) return qpgpu_fail(c, QPGPU_ERR_ARG, "bad u_0_H_u_0 arguments");
  const int64_t N = c->N;
  const size_t cols = (size_t)N * n_st;
  Lock l(c->mu);
  if (c->stage_bytes < 3 * cols * sizeof(double)) {
    dev_free(c->d_stage);
    c->d_stage = nullptr;
    c->stage_bytes = 0;
    QP_CUDA(c, cudaMalloc((void**)&c->d_stage, 3 * cols * sizeof(double)));
    c->stage_bytes = 3 * cols * sizeof(double);
  }
  double *du = c->d_stage, *dv = du + cols, *ds = du + 2 * cols;
  cudaStream_t st = c->stream;
  const int grid = dot_grid(c);
  double* dpart = nullptr;
  QP_CUDA(c, cudaMalloc((void**)&dpart, (size_t)grid * n_st * 2 * sizeof(double)));
  std::vector<double> part((size_t)grid * n_st * 2);
  int* bad = nullptr;
  int hbad = 0;
  rc = qp_numeric_flag(c, st, &bad);
  if (!rc && cudaMemcpy2DAsync(du, N * sizeof(double), u0, ld * sizeof(double), N * sizeof(double), n_st,
                               cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = qpgpu_fail(c, QPGPU_ERR_CUDA, "copy of u_0 failed");
  if (!rc) rc = h_s2_u0_dev(c, dv, ds, du, n_st, N, QPGPU_FP64, st, bad);
  if (!rc) {
    k_col_dots<<<grid, DOT_CTA, 0, st>>>(du, dv, N, n_st, dpart);
    if (cudaMemcpyAsync(part.data(), dpart, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      rc = qpgpu_fail(c, QPGPU_ERR_CUDA, "copy of the dot products failed");
  }
  const cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(dpart);
  if (!rc && e != cudaSuccess) rc = qpgpu_fail(c, QPGPU_ERR_CUDA, cudaGetErrorString(e));
  if (!rc && hbad) rc = qpgpu_fail(c, QPGPU_ERR_NUMERIC, "u_0 holds a NaN or an infinity");
  if (rc) return rc;
  for (int i = 0; i < n_st; ++i) {
    double uu = 0.0, uv = 0.0;
    for (int q = 0; q < grid; ++q) {
      uu += part[((size_t)q * n_st + i) * 2];
      uv += part[((size_t)q * n_st + i) * 2 + 1];
    }
    e_0[i] = (uu != 0.0) ? uv : 0.0;  // the reference's test on u_dot_u; no division (:470-477)
  }
  return QPGPU_OK;
}

int qpgpu_h_s2_u0_work(qpgpu_ctx* c, double* v_t, double* s_t, const double* u_t, int n_st, int istart, int iend,
                       int ishift, int istep) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  if (!v_t || !s_t || !u_t || n_st < 1 || n_st > 8 || istart < 1 || iend > c->N || istep < 1 || ishift < 0)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "bad h_s2_u0_work arguments");
  Lock l(c->mu);
  const int64_t N = c->N;
  const size_t cnt = (size_t)N * n_st;
  double* buf = nullptr;
  QP_CUDA(c, cudaMalloc((void**)&buf, 3 * cnt * sizeof(double)));
  cudaStream_t st = c->stream;
  std::vector<double> hv(cnt), hs(cnt);
  rc = 0;
  if (cudaMemcpyAsync(buf, u_t, cnt * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = qpgpu_fail(c, QPGPU_ERR_CUDA, "copy of u_t failed");
  const int first = istart - 1 + ishift;
  int* bad = nullptr;
  int hbad = 0;
  if (!rc) rc = qp_numeric_flag(c, st, &bad);
  if (!rc) qp_flag_nonfinite(buf, (int64_t)cnt, bad, st);
  if (!rc) rc = qp_sigma_launch(c, &c->items, buf + cnt, buf + 2 * cnt, buf, nullptr, n_st, QPGPU_FP64, st, first,
                                iend, first, istep);
  if (!rc && cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    rc = qpgpu_fail(c, QPGPU_ERR_CUDA, "copy of the NaN flag failed");
  if (!rc && (cudaMemcpyAsync(hv.data(), buf + cnt, cnt * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(hs.data(), buf + 2 * cnt, cnt * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess))
    rc = qpgpu_fail(c, QPGPU_ERR_CUDA, "copy of v_t/s_t failed");
  cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (!rc && e != cudaSuccess) rc = qpgpu_fail(c, QPGPU_ERR_CUDA, cudaGetErrorString(e));
  if (!rc && hbad) rc = qpgpu_fail(c, QPGPU_ERR_NUMERIC, "u_t holds a NaN or an infinity");
  if (rc) return rc;
  for (int64_t k = first; k < iend; k += istep)
    for (int q = 0; q < n_st; ++q) {
      v_t[k * n_st + q] = hv[k * n_st + q];
      s_t[k * n_st + q] = hs[k * n_st + q];
    }
  return QPGPU_OK;
}

int qpgpu_bilinear_order(qpgpu_ctx* c, int32_t* order) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  if (!order) return QPGPU_ERR_ARG;
  Lock l(c->mu);
  QP_CUDA(c, cudaMemcpyAsync(order, c->d_order, c->N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  QP_CUDA(c, cudaStreamSynchronize(c->stream));
  return QPGPU_OK;
}

int qpgpu_diag(qpgpu_ctx* c, double* h_jj, double* s_jj) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  Lock l(c->mu);
  const int64_t N = c->N;
  double* buf = nullptr;
  QP_CUDA(c, cudaMalloc((void**)&buf, 2 * N * sizeof(double)));
  cudaStream_t st = c->stream;
  qp_from_bilinear(c->d_hdiag, N, c->d_order, buf, 1, N, st);
  qp_from_bilinear(c->d_sdiag, N, c->d_order, buf + N, 1, N, st);
  rc = 0;
  if (h_jj && cudaMemcpyAsync(h_jj, buf, N * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = -1;
  if (s_jj && cudaMemcpyAsync(s_jj, buf + N, N * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = -1;
  cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (rc || e != cudaSuccess) return qpgpu_fail(c, QPGPU_ERR_CUDA, "diag copy failed");
  return QPGPU_OK;
}

int qpgpu_connected_pairs(qpgpu_ctx* c, int64_t* n_pairs, int32_t* I, int32_t* J, int8_t* cls, int8_t* phase,
                          int16_t* exc, double* hij, int64_t cap) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  if (!n_pairs) return QPGPU_ERR_ARG;
  Lock l(c->mu);
  if (c->direct) return qpgpu_fail(c, QPGPU_ERR_STATE, "pairs are not stored (direct sigma)");
  *n_pairs = c->P;
  if (cap <= 0) return QPGPU_OK;
  if (cap < c->P || !I || !J || !cls || !phase || !exc || !hij)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "connected_pairs: cap below n_pairs or null output");
  const int64_t P = c->P;
  char* buf = nullptr;
  const size_t bytes = P * (4 + 4 + 1 + 1 + 8 + 8) + 64;
  QP_CUDA(c, cudaMalloc((void**)&buf, bytes));
  int32_t* dI = (int32_t*)buf;
  int32_t* dJ = dI + P;
  double* dh = (double*)(((uintptr_t)(dJ + P) + 15) & ~(uintptr_t)15);
  int16_t* dx = (int16_t*)(dh + P);
  int8_t* dc = (int8_t*)(dx + 4 * P);
  int8_t* dp = dc + P;
  cudaStream_t st = c->stream;
  if (c->nint == 1)
    k_export_pairs<1><<<gsz(P), 256, 0, st>>>(c->tab, c->d_alpha, c->d_beta, c->d_rows, c->d_cols, c->d_order,
                                              c->d_rowptr, c->d_colidx, c->d_val64, c->N, P, dI, dJ, dc, dp, dx, dh);
  else
    k_export_pairs<2><<<gsz(P), 256, 0, st>>>(c->tab, c->d_alpha, c->d_beta, c->d_rows, c->d_cols, c->d_order,
                                              c->d_rowptr, c->d_colidx, c->d_val64, c->N, P, dI, dJ, dc, dp, dx, dh);
  rc = 0;
  if (cudaMemcpyAsync(I, dI, P * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(J, dJ, P * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(hij, dh, P * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(exc, dx, P * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(cls, dc, P, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(phase, dp, P, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    rc = -1;
  cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (rc || e != cudaSuccess) return qpgpu_fail(c, QPGPU_ERR_CUDA, "connected_pairs copy failed");
  return QPGPU_OK;
}

int qpgpu_connected_pairs_rows(qpgpu_ctx* c, const int32_t* rows, int64_t n_rows, int64_t* n_pairs, int32_t* I,
                               int32_t* J, int8_t* cls, int8_t* phase, int16_t* exc, double* hij, int64_t cap) {
  int rc = check_ctx(c, true, true);
  if (rc) return rc;
  if (!n_pairs || n_rows < 0 || (n_rows > 0 && !rows)) return qpgpu_fail(c, QPGPU_ERR_ARG, "bad row list");
  Lock l(c->mu);
  if (c->direct) return qpgpu_fail(c, QPGPU_ERR_STATE, "pairs are not stored (direct sigma)");
  const int64_t N = c->N;
  for (int64_t i = 0; i < n_rows; ++i)
    if (rows[i] < 0 || rows[i] >= N) return qpgpu_fail(c, QPGPU_ERR_ARG, "row index outside 0..N_det-1");
  cudaStream_t st = c->stream;
  std::vector<int> order(N);
  std::vector<int64_t> rowptr(N + 1);
  QP_CUDA(c, cudaMemcpyAsync(order.data(), c->d_order, N * sizeof(int), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaMemcpyAsync(rowptr.data(), c->d_rowptr, (N + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  std::vector<int> inv(N);
  for (int64_t k = 0; k < N; ++k) inv[order[k]] = (int)k;
  std::vector<int> sel((size_t)n_rows);
  for (int64_t i = 0; i < n_rows; ++i) sel[i] = inv[rows[i]];
  std::sort(sel.begin(), sel.end());
  sel.erase(std::unique(sel.begin(), sel.end()), sel.end());
  std::vector<int64_t> beg(sel.size() + 1, 0);
  for (size_t b = 0; b < sel.size(); ++b) beg[b + 1] = beg[b] + (rowptr[sel[b] + 1] - rowptr[sel[b]]);
  const int64_t P = beg.back();
  *n_pairs = P;
  if (cap <= 0 || sel.empty()) return QPGPU_OK;
  if (cap < P || !I || !J || !cls || !phase || !exc || !hij)
    return qpgpu_fail(c, QPGPU_ERR_ARG, "connected_pairs_rows: cap below n_pairs or null output");
  char* buf = nullptr;
  const size_t bytes = P * (4 + 4 + 1 + 1 + 8 + 8) + sel.size() * (4 + 8) + 128;
  QP_CUDA(c, cudaMalloc((void**)&buf, bytes));
  double* dh = (double*)buf;
  int64_t* dbeg = (int64_t*)(dh + P);
  int32_t* dI = (int32_t*)(dbeg + sel.size());
  int32_t* dJ = dI + P;
  int32_t* dsel = dJ + P;
  int16_t* dx = (int16_t*)(dsel + sel.size());
  int8_t* dc = (int8_t*)(dx + 4 * P);
  int8_t* dp = dc + P;
  rc = 0;
  if (cudaMemcpyAsync(dsel, sel.data(), sel.size() * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(dbeg, beg.data(), sel.size() * 8, cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = -1;
  const PairOut out{dI, dJ, dc, dp, dx, dh};
  const unsigned grid = (unsigned)std::min<size_t>(sel.size(), 65535);
  if (!rc) {
    if (c->nint == 1)
      k_export_rows<1><<<grid, 256, 0, st>>>(c->tab, c->d_alpha, c->d_beta, c->d_rows, c->d_cols, c->d_order,
                                             c->d_rowptr, c->d_colidx, c->d_val64, dsel, dbeg, (int)sel.size(), out);
    else
      k_export_rows<2><<<grid, 256, 0, st>>>(c->tab, c->d_alpha, c->d_beta, c->d_rows, c->d_cols, c->d_order,
                                             c->d_rowptr, c->d_colidx, c->d_val64, dsel, dbeg, (int)sel.size(), out);
    if (cudaGetLastError() != cudaSuccess) rc = -1;
  }
  if (!rc && (cudaMemcpyAsync(I, dI, P * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(J, dJ, P * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(hij, dh, P * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(exc, dx, P * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(cls, dc, P, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(phase, dp, P, cudaMemcpyDeviceToHost, st) != cudaSuccess))
    rc = -1;
  cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (rc || e != cudaSuccess) return qpgpu_fail(c, QPGPU_ERR_CUDA, "connected_pairs_rows export failed");
  return QPGPU_OK;
}

}  // extern "C"
