// Hartree-Fock and normal ordering, the input preparation before the flow
// (calc_HF / calc_HO / sqop_to_HF, src/HF_mod.f90:14-209; normal_order,
// src/basic_IMSRG.f90:2419-2550).
//
// Split between host and device:
//  * the mean field of a density, gamma_matrix (src/HF_mod.f90:242-305), is linear in the
//    density: Gamma_B(x,y) = sum M[(B,x,y),(B',g,h)] rho_B'(h,g) / ((j_B+1)(j_B'+1)) with
//    M = sum_J (J+1) V_J(x g, y h).  One device pass over the two-body slab builds M for every
//    pair of orbits sharing (l, j, tz) against every such pair of a block that holds a hole
//    (512 x 172 entries at eMax=10);
//  * the self-consistency loop is tiny (blocks of at most eMax/2+1 orbits) and runs on the
//    host in FP64 with a cyclic Jacobi eigensolver;
//  * the two-body basis change (transform_2b_to_HF, src/HF_mod.f90:567-692) runs on the
//    device.  The reference multiplies dense nt x nt channel matrices (8 nt^3 per channel).
//    Because D only mixes orbits of one (l, j, tz) block, the channel matrix splits into
//    sub-blocks of pairs (a in B1, b in B2) x (c in B3, d in B4); in the unnormalised ordered
//    pair representation V_A(ab,cd) (what v_elem returns) the change of basis of one sub-block
//    is the four-index product D_B1 (x) D_B2 (x) D_B3 (x) D_B4, applied one index at a time in
//    shared memory.  Each stored element is read and written once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "engine.h"
#include "linalg.h"
#include "pair_groups.h"

using namespace imsrg;

// device view of the Hartree-Fock tables
struct HFDev {
  const int* spb_start;  // [nspb] first entry in spb_orb
  const int* spb_n;      // [nspb] orbits in the block
  const int* spb_orb;    // orbits of each block, ascending
  const int* dp_off;     // [nspb] offset of the block's D in the packed coefficients
  const int* grp_b1;     // [ngroups] first sp block of a pair group (b1 <= b2)
  const int* grp_b2;
  const int4* tasks;     // (channel q, group 1, group 2, unused), group 1 <= group 2
  const int* mrow_i;     // mean-field tensor rows: orbit pairs (i, j) of one block
  const int* mrow_j;
  const int* mcol_g;     // columns: orbit pairs (g, h) of one block holding a hole
  const int* mcol_h;
  int nrow, ncol;
};

struct HFState {
  int nspb = 0, nmax = 0;
  std::vector<int> spb_start, spb_n, spb_orb, spb_j, spb_hole, orb_spb, orb_pos, dp_off;
  std::vector<int> row_off, col_off;
  int nrow = 0, ncol = 0, ndp = 0;
  std::vector<int> grp_b1, grp_b2;
  std::vector<int4> tasks;
  HFDev dev{};
  void* tables = nullptr;
  double* d_M = nullptr;
  double* d_dp = nullptr;
  int64_t prefix = 0;  // doubles of the slab before the first two-body array (E0 and f)
};

namespace {

// ---------------------------------------------------------------- device kernels
// M[r + nrow*c] = sum_J (J+1) v_elem(i, g, j, h, J) for row r = (i, j), column c = (g, h)
__global__ void k_hf_mean_field(DevLayout D, HFDev H, const double* op, int herm, double* M) {
  const int64_t n = (int64_t)H.nrow * H.ncol;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % H.nrow), c = (int)(e / H.nrow);
    const int i = H.mrow_i[r], j = H.mrow_j[r], g = H.mcol_g[c], h = H.mcol_h[c];
    const int ji = D.jj[i], jg = D.jj[g];
    double s = 0.0;
    for (int J = abs(ji - jg); J <= ji + jg; J += 2) s += (J + 1) * d_v_elem(D, op, herm, i, g, j, h, J);
    M[e] = s;
  }
}

// out[e] = sum_a C[a + i*n] in[e + (a - i)*stride], i = (e / stride) % n: one index of the
// four-index tensor transformed by the block's coefficient matrix C (column-major n x n)
__device__ __forceinline__ void hf_mode(const double* __restrict__ in, double* __restrict__ out, int ntot, int n,
                                        int stride, const double* __restrict__ C) {
  for (int e = threadIdx.x; e < ntot; e += blockDim.x) {
    const int i = (e / stride) % n;
    const double* src = in + e - i * stride;
    const double* c = C + i * n;
    double s = 0.0;
    for (int a = 0; a < n; ++a) s += c[a] * src[a * stride];
    out[e] = s;
  }
}

// pair (x in block b1, y in block b2) of channel J: stored orbit order, phase, 1/sqrt(1+d)
__device__ __forceinline__ void hf_stored_pair(const DevLayout& D, int oi, int oj, int J, int& lo, int& hi,
                                               double& f) {
  if (oi <= oj) {
    lo = oi; hi = oj;
    f = (oi == oj) ? 0.70710678118654752 : 1.0;
  } else {  // V_A(ji) = -(-1)^((ji+jj-J)/2) V_A(ij)
    lo = oj; hi = oi;
    f = d_sgn(1 + ((D.jj[oi] + D.jj[oj] - J) >> 1));
  }
}

__device__ __forceinline__ void hf_write(const DevLayout& D, double* op, int q, int J, int lo1, int hi1, int lo2,
                                         int hi2, double w) {
  const int C1 = D.con[lo1] + D.con[hi1], C2 = D.con[lo2] + D.con[hi2];
  if (C1 > C2) return;  // the transposed element is stored instead
  const int g = (C1 == 0) ? C2 : (C1 == 1 ? (C2 == 1 ? 3 : 5) : 4);
  const int k = q * 6 + g;
  const int NJ = D.NJ, N = D.N;
  const int i1 = D.pairpos[(lo1 * N + hi1) * NJ + (J >> 1)];
  const int i2 = D.pairpos[(lo2 * N + hi2) * NJ + (J >> 1)];
  op[D.goff[k] + i1 + (int64_t)i2 * D.gn1[k]] = w;
}

// one CTA per (channel, pair group G1 <= G2): gather V_A over the four orbit blocks, apply
// the coefficients index by index, write back every stored element of G1 x G2 and G2 x G1
__global__ void k_hf_transform_2b(DevLayout D, HFDev H, double* op, int herm, const double* __restrict__ dp,
                                  int nmax4) {
  extern __shared__ double hf_sm[];
  double* X = hf_sm;
  double* Y = hf_sm + nmax4;
  const int4 t = H.tasks[blockIdx.x];
  const int q = t.x, G1 = t.y, G2 = t.z;
  const int b[4] = {H.grp_b1[G1], H.grp_b2[G1], H.grp_b1[G2], H.grp_b2[G2]};
  const int n0 = H.spb_n[b[0]], n1 = H.spb_n[b[1]], n2 = H.spb_n[b[2]], n3 = H.spb_n[b[3]];
  const int* o0 = H.spb_orb + H.spb_start[b[0]];
  const int* o1 = H.spb_orb + H.spb_start[b[1]];
  const int* o2 = H.spb_orb + H.spb_start[b[2]];
  const int* o3 = H.spb_orb + H.spb_start[b[3]];
  const int J = D.lamJ[q];
  const int ntot = n0 * n1 * n2 * n3;
  for (int e = threadIdx.x; e < ntot; e += blockDim.x) {
    int r = e;
    const int x0 = r % n0; r /= n0;
    const int x1 = r % n1; r /= n1;
    const int x2 = r % n2;
    const int x3 = r / n2;
    X[e] = d_v_elem(D, op, herm, o0[x0], o1[x1], o2[x2], o3[x3], J);
  }
  __syncthreads();
  hf_mode(X, Y, ntot, n0, 1, dp + H.dp_off[b[0]]);
  __syncthreads();
  hf_mode(Y, X, ntot, n1, n0, dp + H.dp_off[b[1]]);
  __syncthreads();
  hf_mode(X, Y, ntot, n2, n0 * n1, dp + H.dp_off[b[2]]);
  __syncthreads();
  hf_mode(Y, X, ntot, n3, n0 * n1 * n2, dp + H.dp_off[b[3]]);
  __syncthreads();
  // stored pairs of each group: x <= y inside one block, every (x, y) across two blocks
  const bool same1 = b[0] == b[1], same2 = b[2] == b[3];
  const int nbra = same1 ? n0 * (n0 + 1) / 2 : n0 * n1;
  const int nket = same2 ? n2 * (n2 + 1) / 2 : n2 * n3;
  for (int e = threadIdx.x; e < nbra * nket; e += blockDim.x) {
    const int eb = e % nbra, ek = e / nbra;
    int x0, x1, x2, x3;
    if (same1) {
      x1 = 0;
      while ((x1 + 1) * (x1 + 2) / 2 <= eb) ++x1;
      x0 = eb - x1 * (x1 + 1) / 2;
    } else {
      x0 = eb % n0;
      x1 = eb / n0;
    }
    if (same2) {
      x3 = 0;
      while ((x3 + 1) * (x3 + 2) / 2 <= ek) ++x3;
      x2 = ek - x3 * (x3 + 1) / 2;
    } else {
      x2 = ek % n2;
      x3 = ek / n2;
    }
    int lo1, hi1, lo2, hi2;
    double f1, f2;
    hf_stored_pair(D, o0[x0], o1[x1], J, lo1, hi1, f1);
    hf_stored_pair(D, o2[x2], o3[x3], J, lo2, hi2, f2);
    const double v = X[x0 + n0 * (x1 + n1 * (x2 + n2 * x3))] * f1 * f2;
    hf_write(D, op, q, J, lo1, hi1, lo2, hi2, v);
    if (G1 != G2) hf_write(D, op, q, J, lo2, hi2, lo1, hi1, herm * v);
  }
}

// ---------------------------------------------------------------- host helpers
// C = A^T B A for n x n column-major matrices
std::vector<double> sandwich(int n, const std::vector<double>& A, const std::vector<double>& B) {
  std::vector<double> BA((size_t)n * n, 0.0), C((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k)
      for (int i = 0; i < n; ++i) BA[i + (size_t)j * n] += B[i + (size_t)k * n] * A[k + (size_t)j * n];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += A[k + (size_t)i * n] * BA[k + (size_t)j * n];
      C[i + (size_t)j * n] = s;
    }
  return C;
}

}  // namespace

namespace imsrg {

// Symmetric eigenproblem of a small n x n matrix (column-major): cyclic Jacobi with the
// rotation formulas of Rutishauser (Golub and Van Loan, Matrix Computations, sec. 8.5).
// Eigenvalues ascending in w, eigenvectors in the columns of V.
void jacobi_eigen(int n, std::vector<double> A, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i + (size_t)i * n] = 1.0;
  auto a = [&](int i, int j) -> double& { return A[i + (size_t)j * n]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        tot += a(i, j) * a(i, j);
        if (i != j) off += a(i, j) * a(i, j);
      }
    if (off == 0.0 || off <= 1e-34 * tot) break;
    for (int p = 0; p < n - 1; ++p)
      for (int r = p + 1; r < n; ++r) {
        const double apr = a(p, r);
        if (apr == 0.0) continue;
        const double theta = (a(r, r) - a(p, p)) / (2.0 * apr);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- A G (columns p, r)
          const double akp = a(k, p), akr = a(k, r);
          a(k, p) = c * akp - s * akr;
          a(k, r) = s * akp + c * akr;
        }
        for (int k = 0; k < n; ++k) {  // A <- G^T A (rows p, r)
          const double apk = a(p, k), ark = a(r, k);
          a(p, k) = c * apk - s * ark;
          a(r, k) = s * apk + c * ark;
        }
        a(p, r) = a(r, p) = 0.0;
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k + (size_t)p * n], vkr = V[k + (size_t)r * n];
          V[k + (size_t)p * n] = c * vkp - s * vkr;
          V[k + (size_t)r * n] = s * vkp + c * vkr;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
  std::vector<double> Vs((size_t)n * n);
  w.assign(n, 0.0);
  for (int k = 0; k < n; ++k) {
    w[k] = a(idx[k], idx[k]);
    for (int i = 0; i < n; ++i) Vs[i + (size_t)k * n] = V[i + (size_t)idx[k] * n];
  }
  V.swap(Vs);
}

}  // namespace imsrg

#define CKH(expr)                 \
  do {                            \
    imsrg_status _s = (expr);     \
    if (_s != IMSRG_OK) return _s; \
  } while (0)

// sp blocks, mean-field tensor index lists, pair groups and tasks; device copies
imsrg_status Ctx::hf_prepare() {
  if (hf) return IMSRG_OK;
  HFState* S = new (std::nothrow) HFState();
  if (!S) return IMSRG_ERR_OUT_OF_MEMORY;
  hf = S;
  PairGroups PG;
  build_pair_groups(PG, L);
  S->nspb = PG.nspb;
  S->nmax = PG.nmax;
  S->spb_start = PG.spb_start;
  S->spb_n = PG.spb_n;
  S->spb_orb = PG.spb_orb;
  S->spb_j = PG.spb_j;
  S->spb_hole = PG.spb_hole;
  S->orb_spb = PG.orb_spb;
  S->orb_pos = PG.orb_pos;
  S->grp_b1 = PG.grp_b1;
  S->grp_b2 = PG.grp_b2;
  std::vector<int> mri, mrj, mcg, mch;
  for (int B = 0; B < S->nspb; ++B) {
    const int n = S->spb_n[B], s0 = S->spb_start[B];
    S->row_off.push_back(S->nrow);
    S->dp_off.push_back(S->ndp);
    S->ndp += n * n;
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        mri.push_back(S->spb_orb[s0 + x]);
        mrj.push_back(S->spb_orb[s0 + y]);
      }
    S->nrow += n * n;
    if (S->spb_hole[B]) {
      S->col_off.push_back(S->ncol);
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
          mcg.push_back(S->spb_orb[s0 + x]);
          mch.push_back(S->spb_orb[s0 + y]);
        }
      S->ncol += n * n;
    } else {
      S->col_off.push_back(-1);
    }
  }
  // tasks: the group pairs G1 <= G2 of each channel
  for (int q = 0; q < L.nblocks; ++q)
    for (int G2 = PG.grp_first[q]; G2 < PG.grp_first[q + 1]; ++G2)
      for (int G1 = PG.grp_first[q]; G1 <= G2; ++G1) S->tasks.push_back(make_int4(q, G1, G2, 0));
  S->prefix = L.off_fph + (int64_t)L.P * L.A;
  // one device allocation for the integer tables
  std::vector<char> buf;
  auto put = [&](const void* p, size_t bytes) {
    size_t o = (buf.size() + 15) & ~(size_t)15;
    buf.resize(o + bytes);
    if (bytes) std::memcpy(buf.data() + o, p, bytes);
    return o;
  };
  const size_t o_start = put(S->spb_start.data(), sizeof(int) * S->spb_start.size());
  const size_t o_n = put(S->spb_n.data(), sizeof(int) * S->spb_n.size());
  const size_t o_orb = put(S->spb_orb.data(), sizeof(int) * S->spb_orb.size());
  const size_t o_dp = put(S->dp_off.data(), sizeof(int) * S->dp_off.size());
  const size_t o_b1 = put(S->grp_b1.data(), sizeof(int) * S->grp_b1.size());
  const size_t o_b2 = put(S->grp_b2.data(), sizeof(int) * S->grp_b2.size());
  const size_t o_t = put(S->tasks.data(), sizeof(int4) * S->tasks.size());
  const size_t o_ri = put(mri.data(), sizeof(int) * mri.size());
  const size_t o_rj = put(mrj.data(), sizeof(int) * mrj.size());
  const size_t o_cg = put(mcg.data(), sizeof(int) * mcg.size());
  const size_t o_ch = put(mch.data(), sizeof(int) * mch.size());
  CKH(cuda(cudaMalloc(&S->tables, std::max<size_t>(buf.size(), 16)), "cudaMalloc(HF tables)"));
  CKH(cuda(cudaMemcpy(S->tables, buf.data(), buf.size(), cudaMemcpyHostToDevice), "cudaMemcpy(HF tables)"));
  const char* base = (const char*)S->tables;
  S->dev.spb_start = (const int*)(base + o_start);
  S->dev.spb_n = (const int*)(base + o_n);
  S->dev.spb_orb = (const int*)(base + o_orb);
  S->dev.dp_off = (const int*)(base + o_dp);
  S->dev.grp_b1 = (const int*)(base + o_b1);
  S->dev.grp_b2 = (const int*)(base + o_b2);
  S->dev.tasks = (const int4*)(base + o_t);
  S->dev.mrow_i = (const int*)(base + o_ri);
  S->dev.mrow_j = (const int*)(base + o_rj);
  S->dev.mcol_g = (const int*)(base + o_cg);
  S->dev.mcol_h = (const int*)(base + o_ch);
  S->dev.nrow = S->nrow;
  S->dev.ncol = S->ncol;
  CKH(cuda(cudaMalloc(&S->d_M, sizeof(double) * std::max<int64_t>((int64_t)S->nrow * S->ncol, 1)),
           "cudaMalloc(HF mean-field tensor)"));
  CKH(cuda(cudaMalloc(&S->d_dp, sizeof(double) * std::max(S->ndp, 1)), "cudaMalloc(HF coefficients)"));
  const int nmax4 = S->nmax * S->nmax * S->nmax * S->nmax;
  const size_t smem = sizeof(double) * 2 * (size_t)nmax4;
  if (smem > 48 * 1024)
    CKH(cuda(cudaFuncSetAttribute(k_hf_transform_2b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
             "cudaFuncSetAttribute(k_hf_transform_2b)"));
  return IMSRG_OK;
}

void Ctx::hf_release() {
  if (!hf) return;
  for (void* p : {hf->tables, (void*)hf->d_M, (void*)hf->d_dp})
    if (p) cudaFree(p);
  delete hf;
  hf = nullptr;
}

// M of the operator's two-body part, copied to the host
imsrg_status Ctx::hf_mean_field(const double* op, int herm, std::vector<double>& M) {
  HFState& S = *hf;
  const int64_t n = (int64_t)S.nrow * S.ncol;
  M.assign((size_t)n, 0.0);
  if (n == 0) return IMSRG_OK;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
  k_hf_mean_field<<<grid, 256, 0, stream>>>(D, S.dev, op, herm, S.d_M);
  CKH(launched("k_hf_mean_field"));
  CKH(cuda(cudaMemcpyAsync(M.data(), S.d_M, sizeof(double) * n, cudaMemcpyDeviceToHost, stream),
           "cudaMemcpyAsync(HF mean-field tensor)"));
  return cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(HF mean field)");
}

// two-body part of op to the basis of coefs (N x N, D(HO orbit, HF orbit)), in place
imsrg_status Ctx::hf_transform_2b(double* op, int herm, const double* coefs) {
  HFState& S = *hf;
  std::vector<double> dp((size_t)std::max(S.ndp, 1), 0.0);
  for (int B = 0; B < S.nspb; ++B) {
    const int n = S.spb_n[B], s0 = S.spb_start[B];
    for (int i = 0; i < n; ++i)
      for (int a = 0; a < n; ++a)
        dp[S.dp_off[B] + a + i * n] = coefs[S.spb_orb[s0 + a] + (size_t)S.spb_orb[s0 + i] * L.N];
  }
  CKH(cuda(cudaMemcpyAsync(S.d_dp, dp.data(), sizeof(double) * S.ndp, cudaMemcpyHostToDevice, stream),
           "cudaMemcpyAsync(HF coefficients)"));
  if (S.tasks.empty()) return cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(HF)");
  const int nmax4 = S.nmax * S.nmax * S.nmax * S.nmax;
  const size_t smem = sizeof(double) * 2 * (size_t)nmax4;
  const int64_t ntask = (int64_t)S.tasks.size();
  for (int64_t t0 = 0; t0 < ntask; t0 += 2147483647LL) {  // grid.x limit
    const int nb = (int)std::min<int64_t>(ntask - t0, 2147483647LL);
    HFDev dv = S.dev;
    dv.tasks += t0;
    k_hf_transform_2b<<<nb, 128, smem, stream>>>(D, dv, op, herm, S.d_dp, nmax4);
    CKH(launched("k_hf_transform_2b"));
  }
  // the host copy of the coefficients must outlive the copy
  return cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(HF transform)");
}

// mode 0 calc_HF, 1 calc_HO, 2 sqop_to_HF with coefs_in, 3 normal_order
imsrg_status Ctx::hf_run(double* op, int herm, int mode, int max_iter, const double* coefs_in, double* coefs_out,
                         imsrg_hf_info* info) {
  CKH(hf_prepare());
  HFState& S = *hf;
  const int N = L.N, nb = S.nspb;
  std::vector<double> pre((size_t)S.prefix);
  CKH(cuda(cudaMemcpyAsync(pre.data(), op, sizeof(double) * S.prefix, cudaMemcpyDeviceToHost, stream),
           "cudaMemcpyAsync(one-body part)"));
  CKH(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(one-body part)"));
  auto fref = [&](int a, int b) -> double& {  // storage of f(a,b), a, b not (hole, particle)
    if (L.con[a] + L.con[b] == 0) return pre[L.off_fpp + L.loc[a] + (int64_t)L.loc[b] * L.P];
    if (L.con[a] + L.con[b] == 2) return pre[L.off_fhh + L.loc[a] + (int64_t)L.loc[b] * L.A];
    return pre[L.off_fph + L.loc[a] + (int64_t)L.loc[b] * L.P];
  };
  auto f_elem = [&](int a, int b) -> double {  // f_elem (src/basic_IMSRG.f90:1191-1221)
    if (L.con[a] == 1 && L.con[b] == 0) return herm * fref(b, a);
    return fref(a, b);
  };
  auto orb = [&](int B, int x) { return S.spb_orb[S.spb_start[B] + x]; };
  auto upload = [&]() -> imsrg_status {
    CKH(cuda(cudaMemcpyAsync(op, pre.data(), sizeof(double) * S.prefix, cudaMemcpyHostToDevice, stream),
             "cudaMemcpyAsync(one-body part)"));
    return cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(one-body part)");
  };
  // mean field of the block densities rho[B'] (n' x n', scaled by 2j+1), from M
  std::vector<double> M;
  auto gamma = [&](const std::vector<std::vector<double>>& rho, std::vector<std::vector<double>>& G) {
    for (int B = 0; B < nb; ++B) {
      const int n = S.spb_n[B];
      G[B].assign((size_t)n * n, 0.0);
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
          const int64_t r = S.row_off[B] + x + y * n;
          double sm = 0.0;
          for (int B2 = 0; B2 < nb; ++B2) {
            if (S.col_off[B2] < 0) continue;
            const int n2 = S.spb_n[B2];
            double s2 = 0.0;
            for (int h = 0; h < n2; ++h)
              for (int g = 0; g < n2; ++g)
                s2 += M[r + (int64_t)S.nrow * (S.col_off[B2] + g + h * n2)] * rho[B2][h + (size_t)g * n2];
            sm += s2 / (S.spb_j[B2] + 1.0);
          }
          G[B][x + (size_t)y * n] = sm / (S.spb_j[B] + 1.0);
        }
    }
  };
  std::vector<std::vector<double>> T(nb), Dm(nb), G(nb), rho(nb), eig(nb);
  for (int B = 0; B < nb; ++B) {  // write_kin_matrix (src/HF_mod.f90:211-240)
    const int n = S.spb_n[B];
    T[B].assign((size_t)n * n, 0.0);
    for (int x = 0; x < n; ++x)
      for (int y = x; y < n; ++y) T[B][x + (size_t)y * n] = T[B][y + (size_t)x * n] = f_elem(orb(B, x), orb(B, y));
  }
  // transform_1b_to_HF's remap of F' = D^T F D into the one-body arrays (src/HF_mod.f90:530-560)
  auto write_f = [&](int B, const std::vector<double>& Fp) {
    const int n = S.spb_n[B];
    for (int x = 0; x < n; ++x)
      for (int y = x; y < n; ++y) {
        const int i = orb(B, x), j = orb(B, y);
        const int c1 = L.con[i], c2 = L.con[j];
        if (c1 + c2 != 1) {
          fref(i, j) = fref(j, i) = Fp[x + (size_t)y * n];
        } else if (c2 > c1) {
          fref(i, j) = Fp[x + (size_t)y * n];
        } else {
          fref(j, i) = Fp[y + (size_t)x * n];
        }
      }
  };

  if (mode == 3) {  // normal_order (src/basic_IMSRG.f90:2419-2550)
    CKH(hf_mean_field(op, herm, M));
    for (int B = 0; B < nb; ++B) {
      const int n = S.spb_n[B];
      rho[B].assign((size_t)n * n, 0.0);
      for (int x = 0; x < n; ++x) rho[B][x + (size_t)x * n] = L.con[orb(B, x)] * (S.spb_j[B] + 1.0);
    }
    gamma(rho, G);
    double sm = 0.0;
    for (int i = 0; i < N; ++i) sm += f_elem(i, i) * L.con[i] * (L.jj[i] + 1);
    sm *= 2.0;
    for (int B = 0; B < nb; ++B)
      for (int x = 0; x < S.spb_n[B]; ++x)
        sm += L.con[orb(B, x)] * (S.spb_j[B] + 1.0) * G[B][x + (size_t)x * S.spb_n[B]];
    std::vector<double> old = pre;
    auto f_old = [&](int a, int b) -> double {
      if (L.con[a] == 1 && L.con[b] == 0) return herm * old[L.off_fph + L.loc[b] + (int64_t)L.loc[a] * L.P];
      if (L.con[a] + L.con[b] == 0) return old[L.off_fpp + L.loc[a] + (int64_t)L.loc[b] * L.P];
      if (L.con[a] + L.con[b] == 2) return old[L.off_fhh + L.loc[a] + (int64_t)L.loc[b] * L.A];
      return old[L.off_fph + L.loc[a] + (int64_t)L.loc[b] * L.P];
    };
    pre[0] = sm * 0.5;
    for (int B = 0; B < nb; ++B) {
      const int n = S.spb_n[B];
      for (int x = 0; x < n; ++x)
        for (int y = 0; y < n; ++y) {
          const int a = orb(B, x), b = orb(B, y);
          const double v = f_old(a, b) + G[B][x + (size_t)y * n];
          if (L.con[a] == L.con[b]) {
            if (x <= y) fref(a, b) = fref(b, a) = v;
          } else if (L.con[a] == 0) {
            fref(a, b) = v;  // fph(particle, hole)
          }
        }
    }
    return upload();
  }

  if (mode == 2) {  // sqop_to_HF (src/HF_mod.f90:181-209)
    for (int B = 0; B < nb; ++B) {
      const int n = S.spb_n[B];
      Dm[B].assign((size_t)n * n, 0.0);
      for (int i = 0; i < n; ++i)
        for (int a = 0; a < n; ++a) Dm[B][a + (size_t)i * n] = coefs_in[orb(B, a) + (size_t)orb(B, i) * N];
      write_f(B, sandwich(n, Dm[B], T[B]));
    }
    CKH(upload());
    CKH(hf_transform_2b(op, herm, coefs_in));
    return hf_run(op, herm, 3, 0, nullptr, nullptr, nullptr);
  }

  // calc_HF / calc_HO (src/HF_mod.f90:14-179)
  CKH(hf_mean_field(op, herm, M));
  for (int B = 0; B < nb; ++B) {
    const int n = S.spb_n[B];
    Dm[B].assign((size_t)n * n, 0.0);
    for (int x = 0; x < n; ++x) Dm[B][x + (size_t)x * n] = 1.0;
    eig[B].assign(n, 0.0);
  }
  auto density = [&]() {  // density_matrix (src/HF_mod.f90:419-446)
    for (int B = 0; B < nb; ++B) {
      const int n = S.spb_n[B];
      rho[B].assign((size_t)n * n, 0.0);
      for (int k = 0; k < n; ++k) {
        if (!L.con[orb(B, k)]) continue;
        for (int g = 0; g < n; ++g)
          for (int h = 0; h < n; ++h)
            rho[B][h + (size_t)g * n] += Dm[B][h + (size_t)k * n] * Dm[B][g + (size_t)k * n];
      }
      for (double& v : rho[B]) v *= S.spb_j[B] + 1.0;
    }
  };
  const double conv = (double)1e-6f;  // the reference's default-real literal
  double crit = 10.0;
  int iter = 0;
  if (mode == 0) {
    while (crit > conv) {
      if (iter >= max_iter) {
        if (info) { info->e_hf = 0.0; info->crit = crit; info->iterations = iter; }
        return fail(IMSRG_ERR_NOT_CONVERGED, "Hartree-Fock did not converge within max_iter iterations");
      }
      density();
      gamma(rho, G);
      crit = 0.0;
      for (int B = 0; B < nb; ++B) {
        const int n = S.spb_n[B];
        std::vector<double> F(T[B]), w, V;
        for (size_t k = 0; k < F.size(); ++k) F[k] += G[B][k];
        jacobi_eigen(n, F, w, V);
        double d2 = 0.0;
        for (int k = 0; k < n; ++k) d2 += (eig[B][k] - w[k]) * (eig[B][k] - w[k]);
        crit += std::sqrt(d2);
        Dm[B].swap(V);
        eig[B].swap(w);
      }
      ++iter;
    }
  } else {
    density();
    gamma(rho, G);
    crit = 0.0;
  }
  double E = 0.0;
  for (int B = 0; B < nb; ++B) {
    const int n = S.spb_n[B];
    for (int i = 0; i < n; ++i)  // diagonal-positive sign convention (src/HF_mod.f90:85-90)
      if (Dm[B][i + (size_t)i * n] < 0.0)
        for (int a = 0; a < n; ++a) Dm[B][a + (size_t)i * n] = -Dm[B][a + (size_t)i * n];
    std::vector<double> F(T[B]);
    for (size_t k = 0; k < F.size(); ++k) F[k] += G[B][k];
    write_f(B, sandwich(n, Dm[B], F));
    const std::vector<double> Tp = sandwich(n, Dm[B], T[B]), Gp = sandwich(n, Dm[B], G[B]);
    for (int x = 0; x < n; ++x)  // e_HF (src/HF_mod.f90:449-478)
      E += (Tp[x + (size_t)x * n] + 0.5 * Gp[x + (size_t)x * n]) * L.con[orb(B, x)] * (S.spb_j[B] + 1.0);
  }
  pre[0] = E;
  CKH(upload());
  std::vector<double> Dfull((size_t)N * N, 0.0);
  for (int B = 0; B < nb; ++B) {
    const int n = S.spb_n[B];
    for (int i = 0; i < n; ++i)
      for (int a = 0; a < n; ++a) Dfull[orb(B, a) + (size_t)orb(B, i) * N] = Dm[B][a + (size_t)i * n];
  }
  if (mode == 0) CKH(hf_transform_2b(op, herm, Dfull.data()));  // D = 1 leaves calc_HO's V unchanged
  if (coefs_out) std::memcpy(coefs_out, Dfull.data(), sizeof(double) * Dfull.size());
  if (info) {
    info->e_hf = E;
    info->crit = crit;
    info->iterations = iter;
  }
  return IMSRG_OK;
}

#define HCTX(ptr)                                                                        \
  if (!(ptr)) return IMSRG_ERR_INVALID_ARGUMENT;                                         \
  Ctx* c = reinterpret_cast<Ctx*>(ptr);                                                  \
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)"); \
  {                                                                                      \
    cudaError_t _e = cudaSetDevice(c->device);                                           \
    if (_e != cudaSuccess) return c->cuda(_e, "cudaSetDevice");                          \
  }

extern "C" {

imsrg_status imsrg_calc_hf(imsrg_ctx* ctx, imsrg_op* H, int32_t max_iter, double* coefs, imsrg_hf_info* info) {
  HCTX(ctx);
  if (!H || H->owner != c || H->herm != 1 || max_iter < 1)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_calc_hf: hermitian operator of this context, max_iter >= 1");
  return c->hf_run(H->d, 1, 0, max_iter, nullptr, coefs, info);
}

imsrg_status imsrg_calc_ho(imsrg_ctx* ctx, imsrg_op* H, double* coefs, imsrg_hf_info* info) {
  HCTX(ctx);
  if (!H || H->owner != c || H->herm != 1)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_calc_ho: hermitian operator of this context");
  return c->hf_run(H->d, 1, 1, 0, nullptr, coefs, info);
}

imsrg_status imsrg_sqop_to_hf(imsrg_ctx* ctx, imsrg_op* op, const double* coefs) {
  HCTX(ctx);
  if (!op || op->owner != c || !coefs) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_sqop_to_hf");
  return c->hf_run(op->d, op->herm, 2, 0, coefs, nullptr, nullptr);
}

imsrg_status imsrg_transform_2b_to_hf(imsrg_ctx* ctx, imsrg_op* op, const double* coefs) {
  HCTX(ctx);
  if (!op || op->owner != c || !coefs) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_transform_2b_to_hf");
  CKH(c->hf_prepare());
  return c->hf_transform_2b(op->d, op->herm, coefs);
}

imsrg_status imsrg_normal_order(imsrg_ctx* ctx, imsrg_op* op) {
  HCTX(ctx);
  if (!op || op->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_normal_order");
  return c->hf_run(op->d, op->herm, 3, 0, nullptr, nullptr, nullptr);
}

}  // extern "C"
