// Dressed sigma of the MRCC / MRCEPA0 plugins: H_S2_u_0_mrcc_nstates
// (plugins/MRCC_Utils/davidson.irp.f:955-1127) is the sigma of H plus a
// dressing that couples every reference determinant i = idx_ref(ii) with every
// non-reference determinant j = idx_non_ref(jj) through delta_ij(istate,jj,ii)
// -- added both ways, v_i += delta u_j and v_j += delta u_i (:1084-1105), with
// delta_ij_s2 on the S^2 side -- and a diagonal dressing delta_ii(istate,ii)
// added to H_jj of the reference determinants (davidson_diag_mrcc_hs2,
// :547-549), which the sigma's diagonal term then carries (:1120-1124).
//
// The dressing of one state is held on the device with the determinant
// indices mapped to bilinear positions; qp_dress adds it to a sigma already
// computed in the bilinear layout (states fastest).  Two kernels, no atomics:
// one block per reference determinant reduces its row (a sum over all
// non-reference determinants, fixed order), and one thread per non-reference
// determinant adds its column (a short sum over the references).
#include <algorithm>
#include <vector>

#include "qpgpu_internal.cuh"

namespace {

constexpr int RBLK = 256;

// v[ref_ii] += sum_jj d[jj, ii] u[nref_jj] + dii[ii] u[ref_ii]; same for s
// with ds (no diagonal term).  Block per (ii); lanes over jj, then a fixed
// tree over the block.
__global__ void __launch_bounds__(RBLK) k_dress_ref(const int* ref, const int* nref, int64_t n_nref, int n_ref,
                                                    const double* d, const double* ds, const double* dii,
                                                    const double* u, double* v, double* s, int nst) {
  __shared__ double red[2][RBLK];
  for (int ii = blockIdx.x; ii < n_ref; ii += gridDim.x) {
    const double* dcol = d + (int64_t)ii * n_nref;
    const double* scol = ds + (int64_t)ii * n_nref;
    const int64_t ri = ref[ii];
    for (int st = 0; st < nst; ++st) {
      double a = 0.0, b = 0.0;
      for (int64_t jj = threadIdx.x; jj < n_nref; jj += RBLK) {
        const double x = u[(int64_t)nref[jj] * nst + st];
        a = fma(dcol[jj], x, a);
        b = fma(scol[jj], x, b);
      }
      red[0][threadIdx.x] = a;
      red[1][threadIdx.x] = b;
      __syncthreads();
      for (int o = RBLK / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
          red[0][threadIdx.x] += red[0][threadIdx.x + o];
          red[1][threadIdx.x] += red[1][threadIdx.x + o];
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        v[ri * nst + st] += red[0][0] + dii[ii] * u[ri * nst + st];
        s[ri * nst + st] += red[1][0];
      }
      __syncthreads();
    }
  }
}

// v[nref_jj] += sum_ii d[jj, ii] u[ref_ii]; same for s
__global__ void k_dress_nref(const int* ref, const int* nref, int64_t n_nref, int n_ref, const double* d,
                             const double* ds, const double* u, double* v, double* s, int nst) {
  for (int64_t jj = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; jj < n_nref; jj += (int64_t)gridDim.x * blockDim.x) {
    const int64_t rj = nref[jj];
    for (int st = 0; st < nst; ++st) {
      double a = 0.0, b = 0.0;
      for (int ii = 0; ii < n_ref; ++ii) {
        const double x = u[(int64_t)ref[ii] * nst + st];
        a = fma(d[(int64_t)ii * n_nref + jj], x, a);
        b = fma(ds[(int64_t)ii * n_nref + jj], x, b);
      }
      v[rj * nst + st] += a;
      s[rj * nst + st] += b;
    }
  }
}

// hdress (a copy of H_jj) += dii at the reference positions
__global__ void k_dress_diag_ref(double* hdress, const int* ref, const double* dii, int n_ref) {
  for (int ii = blockIdx.x * blockDim.x + threadIdx.x; ii < n_ref; ii += gridDim.x * blockDim.x)
    hdress[ref[ii]] += dii[ii];
}

inline unsigned gsz(int64_t n, int tpb = 256) {
  int64_t g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (unsigned)g;
}

}  // namespace

void qp_free_dressing(qpgpu_ctx* c) {
  Dressing& D = c->dress;
  void* ps[] = {D.ref, D.nref, D.d, D.ds, D.dii, D.hdress};
  for (void* p : ps)
    if (p) cudaFree(p);
  D = Dressing{};
}

int qp_dress(qpgpu_ctx* c, double* v, double* s, const double* u, int nst, cudaStream_t st) {
  const Dressing& D = c->dress;
  if (!D.on) return 0;
  if (D.n_ref > 0)
    k_dress_ref<<<(unsigned)std::min(D.n_ref, 65535), RBLK, 0, st>>>(D.ref, D.nref, D.n_nref, D.n_ref, D.d, D.ds,
                                                                    D.dii, u, v, s, nst);
  if (D.n_nref > 0)
    k_dress_nref<<<gsz(D.n_nref), 256, 0, st>>>(D.ref, D.nref, D.n_nref, D.n_ref, D.d, D.ds, u, v, s, nst);
  QP_CUDA(c, cudaGetLastError());
  return 0;
}

extern "C" int qpgpu_set_dressing(qpgpu_ctx* c, int n_ref, const int32_t* idx_ref, int64_t n_non_ref,
                                  const int32_t* idx_non_ref, const double* delta_ij, const double* delta_ij_s2,
                                  const double* delta_ii) {
  if (!c) return QPGPU_ERR_ARG;
  if (!c->have_pairs) return qpgpu_fail(c, QPGPU_ERR_STATE, "determinants not set");
  if (n_ref < 0 || n_non_ref < 0 || (n_ref > 0 && !idx_ref) || (n_non_ref > 0 && !idx_non_ref) ||
      (n_ref > 0 && n_non_ref > 0 && (!delta_ij || !delta_ij_s2)))
    return qpgpu_fail(c, QPGPU_ERR_ARG, "bad dressing arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  const int64_t N = c->N;
  std::vector<char> seen(N, 0);
  for (int i = 0; i < n_ref; ++i) {
    if (idx_ref[i] < 0 || idx_ref[i] >= N || seen[idx_ref[i]])
      return qpgpu_fail(c, QPGPU_ERR_ARG, "reference indices must be distinct, in 0..N_det-1");
    seen[idx_ref[i]] = 1;
  }
  for (int64_t j = 0; j < n_non_ref; ++j) {
    if (idx_non_ref[j] < 0 || idx_non_ref[j] >= N || seen[idx_non_ref[j]])
      return qpgpu_fail(c, QPGPU_ERR_ARG, "non-reference indices must be distinct, in 0..N_det-1, not references");
    seen[idx_non_ref[j]] = 2;
  }
  qp_free_dressing(c);
  // psi_det index -> bilinear position
  std::vector<int> order(N), inv(N);
  cudaStream_t st = c->stream;
  QP_CUDA(c, cudaMemcpyAsync(order.data(), c->d_order, N * sizeof(int), cudaMemcpyDeviceToHost, st));
  QP_CUDA(c, cudaStreamSynchronize(st));
  for (int64_t k = 0; k < N; ++k) inv[order[k]] = (int)k;
  std::vector<int> ref(n_ref), nref(n_non_ref);
  for (int i = 0; i < n_ref; ++i) ref[i] = inv[idx_ref[i]];
  for (int64_t j = 0; j < n_non_ref; ++j) nref[j] = inv[idx_non_ref[j]];
  Dressing& D = c->dress;
  const size_t nd = (size_t)n_ref * n_non_ref;
  if (dev_alloc(&D.ref, n_ref + 1) != cudaSuccess || dev_alloc(&D.nref, n_non_ref + 1) != cudaSuccess ||
      dev_alloc(&D.d, nd + 1) != cudaSuccess || dev_alloc(&D.ds, nd + 1) != cudaSuccess ||
      dev_alloc(&D.dii, n_ref + 1) != cudaSuccess || dev_alloc(&D.hdress, N) != cudaSuccess) {
    cudaGetLastError();
    qp_free_dressing(c);
    return qpgpu_fail(c, QPGPU_ERR_NOMEM, "dressing does not fit on the device");
  }
  std::vector<double> dii(n_ref, 0.0);
  if (delta_ii)
    for (int i = 0; i < n_ref; ++i) dii[i] = delta_ii[i];
  if (n_ref) QP_CUDA(c, cudaMemcpyAsync(D.ref, ref.data(), n_ref * sizeof(int), cudaMemcpyHostToDevice, st));
  if (n_non_ref) QP_CUDA(c, cudaMemcpyAsync(D.nref, nref.data(), n_non_ref * sizeof(int), cudaMemcpyHostToDevice, st));
  if (nd) {
    QP_CUDA(c, cudaMemcpyAsync(D.d, delta_ij, nd * sizeof(double), cudaMemcpyHostToDevice, st));
    QP_CUDA(c, cudaMemcpyAsync(D.ds, delta_ij_s2, nd * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  if (n_ref) QP_CUDA(c, cudaMemcpyAsync(D.dii, dii.data(), n_ref * sizeof(double), cudaMemcpyHostToDevice, st));
  QP_CUDA(c, cudaMemcpyAsync(D.hdress, c->d_hdiag, N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if (n_ref) k_dress_diag_ref<<<gsz(n_ref), 256, 0, st>>>(D.hdress, D.ref, D.dii, n_ref);
  QP_CUDA(c, cudaGetLastError());
  QP_CUDA(c, cudaStreamSynchronize(st));
  D.n_ref = n_ref;
  D.n_nref = n_non_ref;
  D.on = true;
  return QPGPU_OK;
}

extern "C" int qpgpu_clear_dressing(qpgpu_ctx* c) {
  if (!c) return QPGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStreamSynchronize(c->stream);
  qp_free_dressing(c);
  return QPGPU_OK;
}
