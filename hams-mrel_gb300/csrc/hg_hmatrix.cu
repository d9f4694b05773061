// H-matrix compression of the iterative solver's matrix (the reference's
// ISOLV = 2 path, src/HMatrix.f90), as an option of opts.solver = 2: the
// GMRES matrix-vector products then run on dense near-field blocks and
// low-rank far-field blocks instead of the whole matrix.
//
//  - Cluster tree (host): SPLIT_CLUSTER_ITERATIVE (HMatrix.f90:236-381),
//    geometric bisection at the middle of the longest bounding-box side, at
//    most 32 panels per leaf, explicit stack with the left child first;
//    restated step for step so that the permutation and the tree are the
//    reference's.
//  - Block tree (host): BUILD_BLOCK_TREE_ITERATIVE (:390-497), admissible
//    when the centres are more than 2 x the larger diameter apart (and both
//    sides have more than one panel), the blocks in the reference's order.
//  - ACA (device, k_hm_aca): ADD_LOWRANK_BLOCK (:560-750), partially pivoted
//    adaptive cross approximation to 1e-4 with rank at most 50, one CTA per
//    admissible block, entries read from the assembled matrix through the
//    permutation; kept dense where it stops at rank 0 or saves nothing, or
//    where a side has at most 4 panels.  The stopping test uses the exact
//    update of ||U V^H||_F^2 (the reference's cross term reads past V^H's
//    columns when NR > NC, HMatrix.f90:712-719).
//  - Dense blocks (device, k_hm_gather): copied out of the matrix once.
//  - Product (device): HMATVEC (:760-820) for nc columns: the right-hand
//    sides gathered into cluster order, one CTA per block writing its
//    product to a scratch slice, then per row the sum over the blocks that
//    cover its leaf in the reference's block order (deterministic), scaled
//    and scattered back to the original order.
// All arithmetic in double precision, whatever the matrix's precision.
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "hg_linalg.cuh"

namespace hg {
namespace {

constexpr int kHmNleaf = 32;      // NLEAF_DEFAULT
constexpr double kHmEta = 2.0;    // ETA_DEFAULT
constexpr double kHmTol = 1.0e-4; // ACA_TOL
constexpr int kHmRankMax = 50;    // RANK_MAX
constexpr int kHmThreads = 256;
constexpr int kHmColChunk = 16;   // right-hand-side columns per pass of the block product

struct HmBlock {
  int rs, nr, cs, nc;
  int kmax, rank;  // rank > 0: low rank (U, VH); otherwise dense (D)
  long long u, v, d, t;  // offsets: U (nr x kmax, column-major), VH (kmax x nc, row l contiguous), D (nr x nc), scratch rows
};

__device__ __forceinline__ double2 z_ld(const double2* M, long ld, int i, int j) { return M[i + (long)j * ld]; }
__device__ __forceinline__ double2 z_ld(const float2* M, long ld, int i, int j) {
  const float2 v = M[i + (long)j * ld];
  return make_double2(v.x, v.y);
}
__device__ __forceinline__ double2 z_mul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 z_sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 z_cmul(double2 a, double2 b) {  // conj(a) b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 z_div(double2 a, double2 b) {  // Smith
  if (fabs(b.x) >= fabs(b.y)) {
    const double q = b.y / b.x, d = b.x + b.y * q;
    return make_double2((a.x + a.y * q) / d, (a.y - a.x * q) / d);
  }
  const double q = b.x / b.y, d = b.y + b.x * q;
  return make_double2((a.x * q + a.y) / d, (a.y * q - a.x) / d);
}

// The CTA's largest value, smallest index on ties (every thread gets it).
__device__ void hm_argmax(double& v, int& i, double* sv, int* si) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_down_sync(0xffffffffu, v, o);
    const int oi = __shfl_down_sync(0xffffffffu, i, o);
    if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
  }
  if (lane == 0) { sv[warp] = v; si[warp] = i; }
  __syncthreads();
  if (warp == 0) {
    v = lane < nw ? sv[lane] : -2.0;
    i = lane < nw ? si[lane] : INT_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, v, o);
      const int oi = __shfl_down_sync(0xffffffffu, i, o);
      if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
    }
    if (lane == 0) { sv[0] = v; si[0] = i; }
  }
  __syncthreads();
  v = sv[0];
  i = si[0];
  __syncthreads();
}

// The CTA's sum (fixed order; every thread gets it).
__device__ double hm_sum(double x, double* sv) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if (lane == 0) sv[warp] = x;
  __syncthreads();
  if (warp == 0) {
    x = lane < nw ? sv[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sv[0] = x;
  }
  __syncthreads();
  x = sv[0];
  __syncthreads();
  return x;
}

__device__ __forceinline__ double2 warp_zsum(double2 a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
    a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
  }
  return a;
}

// Partially pivoted ACA of the admissible blocks list[blockIdx.x]; scratch
// per list entry at soff: the residual row (nc) then the used-row flags (nr
// ints).
template <typename T>
__global__ void __launch_bounds__(kHmThreads)
k_hm_aca(HmBlock* __restrict__ blks, const int* __restrict__ list, const long long* __restrict__ soff,
         const int* __restrict__ perm, const T* __restrict__ M, long ld, double2* __restrict__ pool,
         double2* __restrict__ scratch) {
  __shared__ double sv[32];
  __shared__ int si[32];
  const int b = list[blockIdx.x];
  const HmBlock B = blks[b];
  const int nr = B.nr, nc = B.nc, kmax = B.kmax, tid = threadIdx.x, bd = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = bd >> 5;
  double2* U = pool + B.u;
  double2* VH = pool + B.v;
  double2* row = scratch + soff[blockIdx.x];
  int* used = reinterpret_cast<int*>(row + nc);
  for (int i = tid; i < nr; i += bd) used[i] = 0;
  __syncthreads();
  double frob = 0.0;
  int rank = 0, pr = 0;
  for (int k = 0; k < kmax; ++k) {
    if (k > 0) {  // the unused row with the largest |U(:, k-1)|
      double bv = -1.0;
      int bi = INT_MAX;
      for (int i = tid; i < nr; i += bd)
        if (!used[i]) {
          const double2 u = U[i + (long)(k - 1) * nr];
          const double m = hypot(u.x, u.y);
          if (m > bv || (m == bv && i < bi)) { bv = m; bi = i; }
        }
      hm_argmax(bv, bi, sv, si);
      if (bv < 0.0) break;  // every row used
      pr = bi;
    }
    if (tid == 0) used[pr] = 1;
    // residual row pr
    const int gi = perm[B.rs + pr];
    double cv = -1.0;
    int ci = INT_MAX;
    for (int j = tid; j < nc; j += bd) {
      double2 r = z_ld(M, ld, gi, perm[B.cs + j]);
      for (int l = 0; l < k; ++l) r = z_sub(r, z_mul(U[pr + (long)l * nr], VH[(long)l * nc + j]));
      row[j] = r;
      const double m = hypot(r.x, r.y);
      if (m > cv || (m == cv && j < ci)) { cv = m; ci = j; }
    }
    hm_argmax(cv, ci, sv, si);  // the pivot column; its barriers also publish row[]
    const double2 pe = row[ci];
    if (hypot(pe.x, pe.y) < 1.0e-30) break;
    // residual column ci -> U(:, k) = column / pivot; VH(k, :) = row
    const int gj = perm[B.cs + ci];
    for (int i = tid; i < nr; i += bd) {
      double2 cval = z_ld(M, ld, perm[B.rs + i], gj);
      for (int l = 0; l < k; ++l) cval = z_sub(cval, z_mul(U[i + (long)l * nr], VH[(long)l * nc + ci]));
      U[i + (long)k * nr] = z_div(cval, pe);
    }
    for (int j = tid; j < nc; j += bd) VH[(long)k * nc + j] = row[j];
    rank = k + 1;
    __syncthreads();
    // ||u_k|| ||v_k||, and the exact update of ||U V^H||_F^2
    double su = 0.0, sw = 0.0;
    for (int i = tid; i < nr; i += bd) {
      const double2 u = U[i + (long)k * nr];
      su += u.x * u.x + u.y * u.y;
    }
    for (int j = tid; j < nc; j += bd) {
      const double2 w = VH[(long)k * nc + j];
      sw += w.x * w.x + w.y * w.y;
    }
    su = hm_sum(su, sv);
    sw = hm_sum(sw, sv);
    const double uv = sqrt(su) * sqrt(sw);
    double cr = 0.0;
    for (int l = warp; l < k; l += nw) {  // 2 Re (u_l^H u_k)(v_k^H v_l), a warp per l
      double2 a = make_double2(0.0, 0.0), c = make_double2(0.0, 0.0);
      for (int i = lane; i < nr; i += 32) {
        const double2 t = z_cmul(U[i + (long)l * nr], U[i + (long)k * nr]);
        a.x += t.x;
        a.y += t.y;
      }
      for (int j = lane; j < nc; j += 32) {
        const double2 t = z_cmul(VH[(long)l * nc + j], VH[(long)k * nc + j]);
        c.x += t.x;
        c.y += t.y;
      }
      a = warp_zsum(a);
      c = warp_zsum(c);
      if (lane == 0) cr += a.x * c.x - a.y * c.y;
    }
    cr = hm_sum(cr, sv);
    frob += uv * uv + 2.0 * cr;
    if (uv < kHmTol * sqrt(fmax(frob, 1.0e-30))) break;
  }
  if (tid == 0) blks[b].rank = rank;
}

// Dense blocks list[blockIdx.x] copied out of the matrix (cluster order).
template <typename T>
__global__ void k_hm_gather(const HmBlock* __restrict__ blks, const int* __restrict__ list, const int* __restrict__ perm,
                            const T* __restrict__ M, long ld, double2* __restrict__ dpool) {
  const HmBlock B = blks[list[blockIdx.x]];
  double2* D = dpool + B.d;
  const long tot = (long)B.nr * B.nc;
  for (long e = threadIdx.x; e < tot; e += blockDim.x) {
    const int i = (int)(e % B.nr), j = (int)(e / B.nr);
    D[e] = z_ld(M, ld, perm[B.rs + i], perm[B.cs + j]);
  }
}

// xp(r, c) = Z(perm[r], c)
__global__ void k_hm_perm_in(int n, int nc, const int* __restrict__ perm, const double2* __restrict__ Z, long ldz,
                             double2* __restrict__ xp) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r < n && c < nc) xp[r + (long)c * n] = Z[perm[r] + (long)c * ldz];
}

// One CTA per block: its product with the right-hand sides into scratch
// rows (nr x nc at B.t * nc); low rank as U (V^H x), V^H x staged in shared memory.
__global__ void __launch_bounds__(kHmThreads)
k_hm_block_mv(const HmBlock* __restrict__ blks, int n, int nc, const double2* __restrict__ pool,
              const double2* __restrict__ dpool, const double2* __restrict__ xp, double2* __restrict__ tmp) {
  __shared__ double2 vt[kHmRankMax * kHmColChunk];
  const HmBlock B = blks[blockIdx.x];
  double2* out = tmp + B.t * nc;
  for (int c0 = 0; c0 < nc; c0 += kHmColChunk) {
    const int cw = min(kHmColChunk, nc - c0);
    if (B.rank > 0) {
      const double2* U = pool + B.u;
      const double2* VH = pool + B.v;
      const int K = B.rank;
      for (int e = threadIdx.x; e < K * cw; e += blockDim.x) {
        const int l = e % K, c = e / K;
        const double2* x = xp + B.cs + (long)(c0 + c) * n;
        const double2* w = VH + (long)l * B.nc;
        double2 s = make_double2(0.0, 0.0);
        for (int j = 0; j < B.nc; ++j) {
          const double2 t = z_mul(w[j], x[j]);
          s.x += t.x;
          s.y += t.y;
        }
        vt[l + c * K] = s;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < B.nr * cw; e += blockDim.x) {
        const int i = e % B.nr, c = e / B.nr;
        double2 s = make_double2(0.0, 0.0);
        for (int l = 0; l < K; ++l) {
          const double2 t = z_mul(U[i + (long)l * B.nr], vt[l + c * K]);
          s.x += t.x;
          s.y += t.y;
        }
        out[i + (long)(c0 + c) * B.nr] = s;
      }
      __syncthreads();
    } else {
      const double2* D = dpool + B.d;
      for (int e = threadIdx.x; e < B.nr * cw; e += blockDim.x) {
        const int i = e % B.nr, c = e / B.nr;
        const double2* x = xp + B.cs + (long)(c0 + c) * n;
        double2 s = make_double2(0.0, 0.0);
        for (int j = 0; j < B.nc; ++j) {
          const double2 t = z_mul(D[i + (long)j * B.nr], x[j]);
          s.x += t.x;
          s.y += t.y;
        }
        out[i + (long)(c0 + c) * B.nr] = s;
      }
    }
  }
}

// W(perm[r], c) = Bin(perm[r], c) + sign * sum over the blocks covering r's
// leaf (build order) of their scratch rows.
__global__ void k_hm_rows(int n, int nc, const int* __restrict__ perm, const int* __restrict__ leaf_of,
                          const int* __restrict__ lstart, const int* __restrict__ lblk, const HmBlock* __restrict__ blks,
                          const double2* __restrict__ tmp, const double2* __restrict__ Bin, long ldb, double sign,
                          double2* __restrict__ W, long ldw) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= n || c >= nc) return;
  const int L = leaf_of[r];
  double2 s = make_double2(0.0, 0.0);
  for (int q = lstart[L]; q < lstart[L + 1]; ++q) {
    const HmBlock& B = blks[lblk[q]];
    const double2 t = tmp[B.t * nc + (r - B.rs) + (long)c * B.nr];
    s.x += t.x;
    s.y += t.y;
  }
  const int o = perm[r];
  double2 w = make_double2(sign * s.x, sign * s.y);
  if (Bin) {
    const double2 b = Bin[o + (long)c * ldb];
    w.x += b.x;
    w.y += b.y;
  }
  W[o + (long)c * ldw] = w;
}

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t cap = 0;
  ~DBuf() { if (p) cudaFree(p); }
  cudaError_t ensure(size_t count) {
    if (count <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc((void**)&p, (count ? count : 1) * sizeof(T));
    if (e == cudaSuccess) cap = count;
    return e;
  }
};

struct Node {
  int start, end, left, right;
  double center[3], diam;
};

}  // namespace

struct HMatrix::Impl {
  int n = 0;
  std::vector<int> perm, leaf_of, lstart, lblk;
  std::vector<HmBlock> blocks;
  DBuf<int> d_perm, d_leaf, d_lstart, d_lblk, d_list, d_used;
  DBuf<HmBlock> d_blocks;
  DBuf<long long> d_soff;
  DBuf<double2> pool, dpool, scratch, xp, tmp;
  long long tmp_rows = 0;
  HMatrixStats st{};
};

HMatrix::HMatrix() : p(new Impl) {}
HMatrix::~HMatrix() { delete p; }

HMatrixStats HMatrix::stats() const { return p->st; }

// SPLIT_CLUSTER_ITERATIVE and BUILD_BLOCK_TREE_ITERATIVE on the host.
static void hm_trees(int n, const double* xyz, std::vector<Node>& tree, std::vector<int>& perm,
                     std::vector<int>& bl_r, std::vector<int>& bl_c, std::vector<char>& bl_adm) {
  std::vector<double> w(3 * (size_t)n);
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) w[3 * (size_t)i + d] = xyz[i + (size_t)d * n];
  perm.resize(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  struct Item { int i0, i1, parent, side; };
  std::vector<Item> stack{{0, n - 1, -1, 0}};
  while (!stack.empty()) {
    const Item it = stack.back();
    stack.pop_back();
    const int size = it.i1 - it.i0 + 1;
    if (size <= 0) continue;
    const int node = (int)tree.size();
    tree.push_back(Node{it.i0, it.i1, -1, -1, {0, 0, 0}, 0});
    if (it.parent >= 0) (it.side == 1 ? tree[it.parent].left : tree[it.parent].right) = node;
    double bmin[3], bmax[3], cs[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < 3; ++d) bmin[d] = bmax[d] = w[3 * (size_t)it.i0 + d];
    for (int j = it.i0; j <= it.i1; ++j)
      for (int d = 0; d < 3; ++d) {
        const double x = w[3 * (size_t)j + d];
        if (x < bmin[d]) bmin[d] = x;
        if (x > bmax[d]) bmax[d] = x;
        cs[d] += x;
      }
    double blen[3];
    for (int d = 0; d < 3; ++d) {
      tree[node].center[d] = cs[d] / (double)size;
      blen[d] = bmax[d] - bmin[d];
    }
    tree[node].diam = std::sqrt(blen[0] * blen[0] + blen[1] * blen[1] + blen[2] * blen[2]);
    if (size <= kHmNleaf) continue;
    int dim = 0;
    if (blen[1] > blen[dim]) dim = 1;
    if (blen[2] > blen[dim]) dim = 2;
    const double split = 0.5 * (bmin[dim] + bmax[dim]);
    int i = it.i0, j = it.i1;
    while (i <= j) {
      if (w[3 * (size_t)i + dim] <= split) {
        ++i;
      } else {
        for (int d = 0; d < 3; ++d) std::swap(w[3 * (size_t)i + d], w[3 * (size_t)j + d]);
        std::swap(perm[i], perm[j]);
        --j;
      }
    }
    int left_end = i - 1;
    if (left_end < it.i0) left_end = it.i0;
    if (left_end >= it.i1) left_end = it.i1 - 1;
    stack.push_back(Item{left_end + 1, it.i1, node, 2});
    stack.push_back(Item{it.i0, left_end, node, 1});
  }
  std::vector<std::pair<int, int>> bs{{0, 0}};
  while (!bs.empty()) {
    const auto rc = bs.back();
    bs.pop_back();
    const Node &R = tree[rc.first], &C = tree[rc.second];
    const int nr = R.end - R.start + 1, nc = C.end - C.start + 1;
    if (nr <= 0 || nc <= 0) continue;
    const double dx = R.center[0] - C.center[0], dy = R.center[1] - C.center[1], dz = R.center[2] - C.center[2];
    const double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (dist > kHmEta * std::max(R.diam, C.diam) && nr > 1 && nc > 1) {
      bl_r.push_back(rc.first);
      bl_c.push_back(rc.second);
      bl_adm.push_back(1);
      continue;
    }
    const bool lr = R.left < 0, lc = C.left < 0;
    if (lr && lc) {
      bl_r.push_back(rc.first);
      bl_c.push_back(rc.second);
      bl_adm.push_back(0);
      continue;
    }
    if (lr) {
      bs.push_back({rc.first, C.right});
      bs.push_back({rc.first, C.left});
    } else if (lc) {
      bs.push_back({R.right, rc.second});
      bs.push_back({R.left, rc.second});
    } else {
      bs.push_back({R.right, C.right});
      bs.push_back({R.right, C.left});
      bs.push_back({R.left, C.right});
      bs.push_back({R.left, C.left});
    }
  }
}

template <typename T>
static cudaError_t hm_build(HMatrix::Impl* p, cudaStream_t st, int n, const T* M, long ld, const double* xyz) {
  std::vector<Node> tree;
  std::vector<int> br, bc;
  std::vector<char> adm;
  p->n = n;
  p->perm.clear();
  p->blocks.clear();
  hm_trees(n, xyz, tree, p->perm, br, bc, adm);
  const int nb = (int)br.size();
  p->blocks.resize(nb);
  std::vector<int> aca;
  std::vector<long long> soff;
  long long pool = 0, scr = 0;
  for (int b = 0; b < nb; ++b) {
    HmBlock& B = p->blocks[b];
    const Node &R = tree[br[b]], &C = tree[bc[b]];
    B.rs = R.start;
    B.nr = R.end - R.start + 1;
    B.cs = C.start;
    B.nc = C.end - C.start + 1;
    B.rank = 0;
    B.kmax = 0;
    B.u = B.v = B.d = -1;
    if (adm[b] && B.nr > 4 && B.nc > 4) {
      B.kmax = std::min(kHmRankMax, std::min(B.nr, B.nc));
      B.u = pool;
      pool += (long long)B.nr * B.kmax;
      B.v = pool;
      pool += (long long)B.kmax * B.nc;
      aca.push_back(b);
      soff.push_back(scr);
      scr += B.nc + (B.nr + 3) / 4 + 1;  // the row (nc), then nr int flags (4 per double2)
    }
  }
  cudaError_t e;
  if ((e = p->d_perm.ensure(n)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(p->d_perm.p, p->perm.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  if ((e = p->d_blocks.ensure(nb)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(p->d_blocks.p, p->blocks.data(), (size_t)nb * sizeof(HmBlock), cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return e;
  // ACA of the admissible blocks; the ranks come back to decide dense or low rank
  if (!aca.empty()) {
    if ((e = p->pool.ensure((size_t)pool)) != cudaSuccess) return e;
    if ((e = p->scratch.ensure((size_t)scr)) != cudaSuccess) return e;
    if ((e = p->d_list.ensure(aca.size())) != cudaSuccess) return e;
    if ((e = p->d_soff.ensure(soff.size())) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(p->d_list.p, aca.data(), aca.size() * sizeof(int), cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return e;
    if ((e = cudaMemcpyAsync(p->d_soff.p, soff.data(), soff.size() * sizeof(long long), cudaMemcpyHostToDevice, st)) !=
        cudaSuccess)
      return e;
    k_hm_aca<T><<<(int)aca.size(), kHmThreads, 0, st>>>(p->d_blocks.p, p->d_list.p, p->d_soff.p, p->d_perm.p, M, ld,
                                                         p->pool.p, p->scratch.p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    std::vector<HmBlock> back(nb);
    if ((e = cudaMemcpyAsync(back.data(), p->d_blocks.p, (size_t)nb * sizeof(HmBlock), cudaMemcpyDeviceToHost, st)) !=
        cudaSuccess)
      return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    for (int b = 0; b < nb; ++b) p->blocks[b].rank = back[b].rank;
  }
  // final kinds (ADD_LOWRANK_BLOCK's fallback), dense storage, scratch rows
  long long dpool = 0, trows = 0;
  std::vector<int> dense;
  HMatrixStats s{};
  for (int b = 0; b < nb; ++b) {
    HmBlock& B = p->blocks[b];
    if (B.rank > 0 && (long long)B.rank * (B.nr + B.nc) >= (long long)B.nr * B.nc) B.rank = 0;
    if (B.rank == 0) {
      B.d = dpool;
      dpool += (long long)B.nr * B.nc;
      dense.push_back(b);
      ++s.ndense;
      s.bytes += 16.0 * B.nr * B.nc;
    } else {
      ++s.nlowrank;
      s.rank_sum += B.rank;
      s.bytes += 16.0 * B.rank * (B.nr + B.nc);
    }
    B.t = trows;
    trows += B.nr;
  }
  s.nblocks = nb;
  p->st = s;
  p->tmp_rows = trows;
  if ((e = p->dpool.ensure((size_t)std::max(dpool, 1LL))) != cudaSuccess) return e;
  if (pool == 0 && (e = p->pool.ensure(1)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(p->d_blocks.p, p->blocks.data(), (size_t)nb * sizeof(HmBlock), cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return e;
  if (!dense.empty()) {
    if ((e = p->d_list.ensure(std::max(dense.size(), aca.size()))) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(p->d_list.p, dense.data(), dense.size() * sizeof(int), cudaMemcpyHostToDevice, st)) !=
        cudaSuccess)
      return e;
    k_hm_gather<T><<<(int)dense.size(), kHmThreads, 0, st>>>(p->d_blocks.p, p->d_list.p, p->d_perm.p, M, ld, p->dpool.p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  // leaves and, per leaf, the blocks covering it (build order)
  std::vector<int> leaf_start;
  for (const Node& nd : tree)
    if (nd.left < 0) leaf_start.push_back(nd.start);
  std::sort(leaf_start.begin(), leaf_start.end());
  const int nleaf = (int)leaf_start.size();
  p->leaf_of.assign(n, 0);
  for (int L = 0; L < nleaf; ++L) {
    const int e1 = L + 1 < nleaf ? leaf_start[L + 1] : n;
    for (int r = leaf_start[L]; r < e1; ++r) p->leaf_of[r] = L;
  }
  std::vector<std::vector<int>> cover(nleaf);
  for (int b = 0; b < nb; ++b) {
    const HmBlock& B = p->blocks[b];
    for (int L = p->leaf_of[B.rs]; L < nleaf && leaf_start[L] < B.rs + B.nr; ++L) cover[L].push_back(b);
  }
  p->lstart.assign(nleaf + 1, 0);
  p->lblk.clear();
  for (int L = 0; L < nleaf; ++L) {
    p->lstart[L] = (int)p->lblk.size();
    p->lblk.insert(p->lblk.end(), cover[L].begin(), cover[L].end());
  }
  p->lstart[nleaf] = (int)p->lblk.size();
  if ((e = p->d_leaf.ensure(n)) != cudaSuccess) return e;
  if ((e = p->d_lstart.ensure(nleaf + 1)) != cudaSuccess) return e;
  if ((e = p->d_lblk.ensure(p->lblk.size())) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(p->d_leaf.p, p->leaf_of.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(p->d_lstart.p, p->lstart.data(), (size_t)(nleaf + 1) * sizeof(int), cudaMemcpyHostToDevice,
                           st)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(p->d_lblk.p, p->lblk.data(), p->lblk.size() * sizeof(int), cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return e;
  return cudaStreamSynchronize(st);  // the host vectors above are copied before they go
}

int hmatrix_partition(int n, const double* xyz, int* perm, int* blocks, int max_blocks) {
  if (n <= 0 || !xyz) return -1;
  std::vector<Node> tree;
  std::vector<int> pm, br, bc;
  std::vector<char> adm;
  hm_trees(n, xyz, tree, pm, br, bc, adm);
  if (perm) std::copy(pm.begin(), pm.end(), perm);
  const int nb = (int)br.size();
  if (blocks)
    for (int b = 0; b < nb && b < max_blocks; ++b) {
      int* o = blocks + 5 * (size_t)b;
      o[0] = tree[br[b]].start;
      o[1] = tree[br[b]].end - tree[br[b]].start + 1;
      o[2] = tree[bc[b]].start;
      o[3] = tree[bc[b]].end - tree[bc[b]].start + 1;
      o[4] = adm[b];
    }
  return nb;
}

size_t hmatrix_bytes_estimate(int n, const double* xyz, int nc) {
  if (n <= 0 || !xyz) return 0;
  std::vector<Node> tree;
  std::vector<int> perm, br, bc;
  std::vector<char> adm;
  hm_trees(n, xyz, tree, perm, br, bc, adm);
  size_t elems = 0, rows = 0;
  for (size_t b = 0; b < br.size(); ++b) {
    const size_t nr = (size_t)(tree[br[b]].end - tree[br[b]].start + 1), ncl = (size_t)(tree[bc[b]].end - tree[bc[b]].start + 1);
    if (adm[b] && nr > 4 && ncl > 4) {
      const size_t kmax = std::min<size_t>(kHmRankMax, std::min(nr, ncl));
      elems += kmax * (nr + ncl) + ncl + (nr + 3) / 4 + 1;  // factors and the ACA scratch
    } else {
      elems += nr * ncl;
    }
    rows += nr;
  }
  elems += rows * (size_t)nc + (size_t)n * nc;  // the product's scratch rows and permuted right-hand sides
  return elems * sizeof(double2) + br.size() * (sizeof(HmBlock) + 2 * sizeof(int)) + (size_t)4 * n * sizeof(int);
}

cudaError_t HMatrix::build(cudaStream_t st, int n, const double2* M, const float2* Mf, long ld, const double* xyz) {
  if (n <= 0 || (!M && !Mf) || !xyz) return cudaErrorInvalidValue;
  return M ? hm_build<double2>(p, st, n, M, ld, xyz) : hm_build<float2>(p, st, n, Mf, ld, xyz);
}

cudaError_t HMatrix::matvec(cudaStream_t st, int nc, const double2* Z, long ldz, const double2* Bin, long ldb,
                            double sign, double2* W, long ldw) {
  const int n = p->n;
  if (n <= 0 || nc <= 0) return n <= 0 ? cudaErrorInvalidValue : cudaSuccess;
  cudaError_t e;
  if ((e = p->xp.ensure((size_t)n * nc)) != cudaSuccess) return e;
  if ((e = p->tmp.ensure((size_t)p->tmp_rows * nc)) != cudaSuccess) return e;
  const dim3 g((n + 255) / 256, nc);
  k_hm_perm_in<<<g, 256, 0, st>>>(n, nc, p->d_perm.p, Z, ldz, p->xp.p);
  k_hm_block_mv<<<(int)p->blocks.size(), kHmThreads, 0, st>>>(p->d_blocks.p, n, nc, p->pool.p, p->dpool.p, p->xp.p,
                                                               p->tmp.p);
  k_hm_rows<<<g, 256, 0, st>>>(n, nc, p->d_perm.p, p->d_leaf.p, p->d_lstart.p, p->d_lblk.p, p->d_blocks.p, p->tmp.p, Bin,
                               ldb, sign, W, ldw);
  return cudaGetLastError();
}

}  // namespace hg
