// bvh.cu -- device construction of the 4-wide BVHs.
//
// Linear BVH (Karras 2012, "Maximizing parallelism in the construction of
// BVHs, octrees and k-d trees"):
//   1. primitive boxes (already dilated by the caller) -> centroid bounds
//   2. 63-bit Morton codes of the centroids (21 bits per axis)
//   3. radix sort of (code, primitive) pairs (CUB, build time only)
//   4. binary radix tree, one thread per inner node; equal codes are split by
//      primitive position so the tree is well formed for duplicates
//   5. bottom-up box refit: one thread per leaf climbs, the second thread to
//      reach a node computes its box (atomic arrival counter)
//   6. collapse to W-wide nodes (W = 4 or 8) top-down, one level per launch,
//      either
//      (a) by the SAH: a bottom-up dynamic program over the binary tree
//          (the optimal wide-BVH conversion of Ylitie, Karras and Laine,
//          "Efficient incoherent ray traversal on GPUs through compressed
//          wide BVHs", HPG 2017) finds, for every binary node and every
//          number of child slots k <= W, the cheapest way to cover its
//          subtree with k slots, each a leaf of <= leaf_max primitives or a
//          wide node, under the cost  sum over wide nodes of area * C_node
//          + sum over leaves of area * primitives * C_prim;  the collapse
//          then reads each wide node's children off the stored decisions;
//      or (b) greedily: a wide node repeatedly opens the child with the
//          largest surface area until it has W children; subtrees with at
//          most leaf_max primitives become leaves.
//      Leaves are binary subtrees, so their primitives are contiguous in
//      sorted order.  An 8-wide node is stored as two consecutive 4-wide
//      records (children 0-3 and 4-7), so node index k occupies records 2k
//      and 2k+1.
// Every loop is bounded by the primitive count; no thread waits on another.
#include <cub/device/device_radix_sort.cuh>

#include <vector>

#include "bvh.h"

namespace xdgcu {

namespace {

__device__ __forceinline__ unsigned long long ord_encode(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

__host__ __forceinline__ double ord_decode(unsigned long long e) {
  unsigned long long b = (e & 0x8000000000000000ull) ? (e & 0x7fffffffffffffffull) : ~e;
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
}

// bounds[0..2] = encoded min centroid, bounds[3..5] = encoded max centroid,
// bounds[6..8] = min box lo, bounds[9..11] = max box hi
__global__ void k_bounds(const double* __restrict__ boxes, int32_t n,
                         unsigned long long* __restrict__ bounds) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  double c[3], lo[3], hi[3];
  bool valid = i < n;
  for (int k = 0; k < 3; ++k) {
    if (valid) {
      lo[k] = boxes[6 * (int64_t)i + k];
      hi[k] = boxes[6 * (int64_t)i + 3 + k];
      c[k] = 0.5 * (lo[k] + hi[k]);
    }
  }
  for (int k = 0; k < 3; ++k) {
    unsigned long long cmin = valid ? ord_encode(c[k]) : ~0ull;
    unsigned long long cmax = valid ? ord_encode(c[k]) : 0ull;
    unsigned long long bmin = valid ? ord_encode(lo[k]) : ~0ull;
    unsigned long long bmax = valid ? ord_encode(hi[k]) : 0ull;
    for (int off = 16; off > 0; off >>= 1) {
      cmin = min(cmin, __shfl_xor_sync(0xffffffffu, cmin, off));
      cmax = max(cmax, __shfl_xor_sync(0xffffffffu, cmax, off));
      bmin = min(bmin, __shfl_xor_sync(0xffffffffu, bmin, off));
      bmax = max(bmax, __shfl_xor_sync(0xffffffffu, bmax, off));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&bounds[k], cmin);
      atomicMax(&bounds[3 + k], cmax);
      atomicMin(&bounds[6 + k], bmin);
      atomicMax(&bounds[9 + k], bmax);
    }
  }
}

__device__ __forceinline__ unsigned long long spread21(unsigned long long x) {
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

__global__ void k_morton(const double* __restrict__ boxes, int32_t n, double3 cmin, double3 cinv,
                         unsigned long long* __restrict__ keys, int32_t* __restrict__ vals) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* b = boxes + 6 * (int64_t)i;
  double q[3] = {(0.5 * (b[0] + b[3]) - cmin.x) * cinv.x, (0.5 * (b[1] + b[4]) - cmin.y) * cinv.y,
                 (0.5 * (b[2] + b[5]) - cmin.z) * cinv.z};
  unsigned long long code = 0;
  for (int k = 0; k < 3; ++k) {
    double s = fmin(fmax(q[k], 0.0), 1.0) * 2097151.0;
    code |= spread21((unsigned long long)s) << (2 - k);
  }
  keys[i] = code;
  vals[i] = i;
}

struct Karras {
  const unsigned long long* keys;
  int32_t n;
  __device__ __forceinline__ int delta(int32_t a, int32_t b) const {
    if (b < 0 || b >= n) return -1;
    unsigned long long ka = keys[a], kb = keys[b];
    if (ka != kb) return __clzll((long long)(ka ^ kb));
    return 64 + __clz(a ^ b);
  }
};

// binary node ids: inner i in [0, n-1), leaf j -> n-1+j
__global__ void k_karras(Karras K, int32_t* __restrict__ left, int32_t* __restrict__ right,
                         int32_t* __restrict__ parent, int32_t* __restrict__ first,
                         int32_t* __restrict__ last) {
  const int32_t n = K.n;
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (K.delta(i, i + 1) - K.delta(i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = K.delta(i, i - d);
  int64_t lmax = 2;
  while (K.delta(i, (int32_t)(i + lmax * d)) > dmin && lmax < 2 * (int64_t)n) lmax *= 2;
  int64_t l = 0;
  for (int64_t t = lmax / 2; t >= 1; t /= 2)
    if (K.delta(i, (int32_t)(i + (l + t) * d)) > dmin) l += t;
  const int32_t j = (int32_t)(i + l * d);
  const int dnode = K.delta(i, j);
  int64_t s = 0;
  for (int64_t div = 2;; div <<= 1) {
    const int64_t t = (l + div - 1) / div;
    if (K.delta(i, (int32_t)(i + (s + t) * d)) > dnode) s += t;
    if (t <= 1) break;
  }
  const int32_t gamma = (int32_t)(i + s * d + (d < 0 ? -1 : 0));
  const int32_t lo = min(i, j), hi = max(i, j);
  const int32_t lc = (lo == gamma) ? (n - 1 + gamma) : gamma;
  const int32_t rc = (hi == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
  left[i] = lc;
  right[i] = rc;
  first[i] = lo;
  last[i] = hi;
  parent[lc] = i;
  parent[rc] = i;
}

__global__ void k_refit(const double* __restrict__ boxes, const int32_t* __restrict__ vals,
                        int32_t n, const int32_t* __restrict__ left,
                        const int32_t* __restrict__ right, const int32_t* __restrict__ parent,
                        int32_t* __restrict__ flag, double* __restrict__ nbox) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int32_t node = n - 1 + j;
  const double* b = boxes + 6 * (int64_t)vals[j];
  for (int k = 0; k < 6; ++k) nbox[6 * (int64_t)node + k] = b[k];
  __threadfence();
  int32_t p = parent[node];
  while (p >= 0) {
    if (atomicAdd(&flag[p], 1) == 0) return;
    __threadfence();
    const int32_t a = left[p], c = right[p];
    double out[6];
    for (int k = 0; k < 3; ++k) {
      out[k] = fmin(__ldcg(&nbox[6 * (int64_t)a + k]), __ldcg(&nbox[6 * (int64_t)c + k]));
      out[3 + k] = fmax(__ldcg(&nbox[6 * (int64_t)a + 3 + k]), __ldcg(&nbox[6 * (int64_t)c + 3 + k]));
    }
    for (int k = 0; k < 6; ++k) __stcg(&nbox[6 * (int64_t)p + k], out[k]);
    __threadfence();
    p = parent[p];
  }
}

struct CollapseArgs {
  const int32_t* left;
  const int32_t* right;
  const int32_t* first;
  const int32_t* last;
  const double* nbox;
  int32_t n;
  int32_t leaf_max;
  Node32* n32;
  Node64* n64;
  int32_t* node_counter;
  int32_t* out_count;
};

__device__ __forceinline__ double half_area(const double* b) {
  const double dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
  return dx * dy + dy * dz + dz * dx;
}

// ---- SAH collapse ------------------------------------------------------
//
// Per binary node c (inner c < n-1, leaf n-1+j) and k = 1..W slots:
//   S[c][k-1]  the least cost of covering c's subtree with at most k slots;
//   dec[c][k-1] for k = 1: 1 when c is best a wide node, 0 a leaf; for k >= 2:
//              0 when S[c][k-1] = S[c][k-2] (fewer slots suffice), else the
//              number of slots j (1..k-1) given to the left child (the rest to
//              the right).
// For a wide node at c the children are the slots of (left, j), (right, W-j)
// with j = split[c], the best division of W slots.
constexpr int kSahW = 8;
constexpr float kInfCost = 3.0e38f;

struct SahArgs {
  const int32_t* left;
  const int32_t* right;
  const int32_t* parent;
  const int32_t* first;
  const int32_t* last;
  const double* nbox;
  int32_t n;
  int32_t leaf_max;
  int32_t width;
  float c_node, c_prim;
  float* S;         // width per binary node
  uint8_t* dec;     // width per binary node
  uint8_t* split;   // per inner node: slots of the left child in a wide node at it
  int32_t* flag;
};

__device__ __forceinline__ float node_area(const double* nbox, int32_t c) {
  const double* b = nbox + 6 * (int64_t)c;
  const double dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
  return (float)(dx * dy + dy * dz + dz * dx);
}

// S and dec of inner node p from its children's tables (already complete).
__device__ void sah_node(const SahArgs& A, int32_t p) {
  const int W = A.width;
  const int32_t l = A.left[p], r = A.right[p];
  float Sl[kSahW], Sr[kSahW];
  for (int k = 0; k < W; ++k) {
    Sl[k] = __ldcg(&A.S[(int64_t)l * W + k]);
    Sr[k] = __ldcg(&A.S[(int64_t)r * W + k]);
  }
  // D[j-1]: best cost of spreading p's subtree over exactly-at-most j >= 2
  // slots, j1[j-1] the left child's share
  float D[kSahW];
  uint8_t j1[kSahW];
  for (int j = 2; j <= W; ++j) {
    float best = kInfCost;
    int bk = 1;
    for (int k = 1; k < j; ++k) {
      const float v = Sl[k - 1] + Sr[j - k - 1];
      if (v < best) {
        best = v;
        bk = k;
      }
    }
    D[j - 1] = best;
    j1[j - 1] = (uint8_t)bk;
  }
  const float area = node_area(A.nbox, p);
  const int32_t cnt = A.last[p] - A.first[p] + 1;
  const float c_leaf = cnt <= A.leaf_max ? area * A.c_prim * (float)cnt : kInfCost;
  const float c_wide = area * A.c_node + D[W - 1];
  float Sp[kSahW];
  uint8_t dp[kSahW];
  Sp[0] = c_leaf <= c_wide ? c_leaf : c_wide;
  dp[0] = c_leaf <= c_wide ? 0 : 1;
  for (int k = 2; k <= W; ++k) {
    if (D[k - 1] < Sp[k - 2]) {
      Sp[k - 1] = D[k - 1];
      dp[k - 1] = j1[k - 1];
    } else {
      Sp[k - 1] = Sp[k - 2];
      dp[k - 1] = 0;
    }
  }
  for (int k = 0; k < W; ++k) {
    __stcg(&A.S[(int64_t)p * W + k], Sp[k]);
    A.dec[(int64_t)p * W + k] = dp[k];
  }
  A.split[p] = j1[W - 1];
}

// Bottom-up over the binary tree, one thread per leaf; the second thread to
// reach a node evaluates it (as k_refit).
__global__ void k_sah(SahArgs A) {
  const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= A.n) return;
  const int W = A.width;
  const int32_t leaf = A.n - 1 + j;
  const float c = node_area(A.nbox, leaf) * A.c_prim;
  for (int k = 0; k < W; ++k) {
    __stcg(&A.S[(int64_t)leaf * W + k], c);
    A.dec[(int64_t)leaf * W + k] = 0;
  }
  __threadfence();
  int32_t p = A.parent[leaf];
  while (p >= 0) {
    if (atomicAdd(&A.flag[p], 1) == 0) return;
    __threadfence();
    sah_node(A, p);
    __threadfence();
    p = A.parent[p];
  }
}

// The children of a wide node at binary node b: the slots of (left, split)
// and (right, W - split), each expanded by the stored decisions.
template <int W>
__device__ int sah_children(const SahArgs& A, int32_t b, int32_t* ch) {
  int32_t sn[2 * W];
  int sk[2 * W];
  int top = 0, cnt = 0;
  const int s = A.split[b];
  sn[top] = A.right[b];
  sk[top++] = W - s;
  sn[top] = A.left[b];
  sk[top++] = s;
  while (top > 0 && cnt < W) {
    int32_t c = sn[--top];
    int k = sk[top];
    while (true) {
      if (c >= A.n - 1 || k <= 1) {  // a binary leaf, or one slot: c itself
        ch[cnt++] = c;
        break;
      }
      const int d = A.dec[(int64_t)c * W + (k - 1)];
      if (d == 0) {  // fewer slots are as cheap
        --k;
        continue;
      }
      if (top + 1 >= 2 * W) {  // cannot happen: each expansion adds one slot
        ch[cnt++] = c;
        break;
      }
      sn[top] = A.right[c];
      sk[top++] = k - d;
      c = A.left[c];
      k = d;
    }
  }
  return cnt;
}

template <int W>
__global__ void k_collapse(CollapseArgs A, const int2* __restrict__ in, int32_t n_in,
                           int2* __restrict__ out, SahArgs sah, int use_sah) {
  int32_t it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= n_in) return;
  const int32_t b = in[it].x, w = in[it].y;
  const int32_t n = A.n;
  auto is_inner = [&](int32_t c) { return c < n - 1; };
  auto count_of = [&](int32_t c) { return is_inner(c) ? A.last[c] - A.first[c] + 1 : 1; };
  int32_t ch[W];
  int cnt = 2;
  ch[0] = A.left[b];
  ch[1] = A.right[b];
  if (use_sah) cnt = sah_children<W>(sah, b, ch);
  while (!use_sah && cnt < W) {
    int best = -1;
    double best_area = -1.0;
    for (int k = 0; k < cnt; ++k) {
      const int32_t c = ch[k];
      if (is_inner(c) && count_of(c) > A.leaf_max) {
        const double a = half_area(A.nbox + 6 * (int64_t)c);
        if (a > best_area) {
          best_area = a;
          best = k;
        }
      }
    }
    if (best < 0) break;
    const int32_t c = ch[best];
    ch[best] = A.left[c];
    ch[cnt++] = A.right[c];
  }
  for (int rec = 0; rec < W / kWidth; ++rec) {
  Node32 n32;
  Node64 n64;
  float* f32[6] = {&n32.lox.x, &n32.hix.x, &n32.loy.x, &n32.hiy.x, &n32.loz.x, &n32.hiz.x};
  double* f64[6] = {n64.lox, n64.hix, n64.loy, n64.hiy, n64.loz, n64.hiz};
  int refs[kWidth];
  for (int kk = 0; kk < kWidth; ++kk) {
    const int k = rec * kWidth + kk;
    if (k < cnt) {
      const int32_t c = ch[k];
      const double* bx = A.nbox + 6 * (int64_t)c;
      for (int a = 0; a < 3; ++a) {
        f64[2 * a][kk] = bx[a];
        f64[2 * a + 1][kk] = bx[3 + a];
        f32[2 * a][kk] = __double2float_rd(bx[a]);
        f32[2 * a + 1][kk] = __double2float_ru(bx[3 + a]);
      }
      const int32_t cc = count_of(c);
      const bool leaf = use_sah ? (!is_inner(c) || sah.dec[(int64_t)c * W] == 0)
                                : (!is_inner(c) || cc <= A.leaf_max);
      if (leaf) {
        const int32_t f = is_inner(c) ? A.first[c] : c - (n - 1);
        refs[kk] = make_leaf(f, cc);
      } else {
        const int32_t nw = atomicAdd(A.node_counter, 1);
        const int32_t slot = atomicAdd(A.out_count, 1);
        out[slot] = make_int2(c, nw);
        refs[kk] = nw;
      }
    } else {
      for (int a = 0; a < 3; ++a) {
        f64[2 * a][kk] = INFINITY;
        f64[2 * a + 1][kk] = -INFINITY;
        f32[2 * a][kk] = INFINITY;
        f32[2 * a + 1][kk] = -INFINITY;
      }
      refs[kk] = CHILD_EMPTY;
    }
  }
  n32.child = make_int4(refs[0], refs[1], refs[2], refs[3]);
  n64.child = n32.child;
  A.n32[(int64_t)w * (W / kWidth) + rec] = n32;
  A.n64[(int64_t)w * (W / kWidth) + rec] = n64;
  }
}

}  // namespace

#define BVH_CHECK(x)                          \
  do {                                        \
    cudaError_t e_ = (x);                     \
    if (e_ != cudaSuccess) return e_;         \
  } while (0)

cudaError_t build_wide_bvh(const double* d_boxes, int32_t n, int32_t leaf_max, int32_t width,
                           const BvhCost* sah_cost, cudaStream_t st, BuiltTree* out) {
  if (width != 4 && width != 8) return cudaErrorInvalidValue;
  out->width = width;
  out->n32 = nullptr;
  out->n64 = nullptr;
  out->order = nullptr;
  out->n_nodes = 0;
  out->depth = 0;
  out->root = CHILD_EMPTY;
  for (int k = 0; k < 6; ++k) out->bounds[k] = 0.0;
  if (n <= 0) return cudaSuccess;
  if (leaf_max < 1) leaf_max = 1;
  if (leaf_max > 16) leaf_max = 16;

  DevMem<unsigned long long> bounds(12);
  std::vector<unsigned long long> hb(12);
  for (int k = 0; k < 3; ++k) {
    hb[k] = ~0ull;
    hb[3 + k] = 0ull;
    hb[6 + k] = ~0ull;
    hb[9 + k] = 0ull;
  }
  BVH_CHECK(bounds.alloc());
  BVH_CHECK(cudaMemcpyAsync(bounds.p, hb.data(), 12 * sizeof(unsigned long long),
                            cudaMemcpyHostToDevice, st));
  const int B = 256;
  const int G = (n + B - 1) / B;
  k_bounds<<<G, B, 0, st>>>(d_boxes, n, bounds.p);
  BVH_CHECK(cudaGetLastError());
  BVH_CHECK(cudaMemcpyAsync(hb.data(), bounds.p, 12 * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, st));
  BVH_CHECK(cudaStreamSynchronize(st));
  double cmin[3], cmax[3];
  for (int k = 0; k < 3; ++k) {
    cmin[k] = ord_decode(hb[k]);
    cmax[k] = ord_decode(hb[3 + k]);
    out->bounds[k] = ord_decode(hb[6 + k]);
    out->bounds[3 + k] = ord_decode(hb[9 + k]);
  }

  BVH_CHECK(cudaMalloc(&out->order, sizeof(int32_t) * n));
  if (n == 1) {
    int32_t zero = 0;
    BVH_CHECK(cudaMemcpyAsync(out->order, &zero, sizeof zero, cudaMemcpyHostToDevice, st));
    BVH_CHECK(cudaStreamSynchronize(st));
    out->root = make_leaf(0, 1);
    return cudaSuccess;
  }

  // Morton codes + sort
  DevMem<unsigned long long> keys(n), keys2(n);
  DevMem<int32_t> vals(n);
  BVH_CHECK(keys.alloc());
  BVH_CHECK(keys2.alloc());
  BVH_CHECK(vals.alloc());
  double3 c0 = make_double3(cmin[0], cmin[1], cmin[2]);
  double3 ci;
  ci.x = cmax[0] > cmin[0] ? 1.0 / (cmax[0] - cmin[0]) : 0.0;
  ci.y = cmax[1] > cmin[1] ? 1.0 / (cmax[1] - cmin[1]) : 0.0;
  ci.z = cmax[2] > cmin[2] ? 1.0 / (cmax[2] - cmin[2]) : 0.0;
  k_morton<<<G, B, 0, st>>>(d_boxes, n, c0, ci, keys.p, vals.p);
  BVH_CHECK(cudaGetLastError());
  size_t tmp_bytes = 0;
  BVH_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.p, keys2.p, vals.p,
                                            out->order, n, 0, 63, st));
  DevMem<char> tmp(tmp_bytes);
  BVH_CHECK(tmp.alloc());
  BVH_CHECK(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.p, keys2.p, vals.p, out->order,
                                            n, 0, 63, st));

  // binary tree
  const int32_t nb = 2 * n - 1;
  DevMem<int32_t> left(n - 1), right(n - 1), first(n - 1), last(n - 1), parent(nb), flag(n - 1);
  DevMem<double> nbox(6 * (int64_t)nb);
  BVH_CHECK(left.alloc());
  BVH_CHECK(right.alloc());
  BVH_CHECK(first.alloc());
  BVH_CHECK(last.alloc());
  BVH_CHECK(parent.alloc());
  BVH_CHECK(flag.alloc());
  BVH_CHECK(nbox.alloc());
  BVH_CHECK(cudaMemsetAsync(parent.p, 0xff, sizeof(int32_t) * nb, st));
  BVH_CHECK(cudaMemsetAsync(flag.p, 0, sizeof(int32_t) * (n - 1), st));
  Karras K{keys2.p, n};
  k_karras<<<(n - 1 + B - 1) / B, B, 0, st>>>(K, left.p, right.p, parent.p, first.p, last.p);
  BVH_CHECK(cudaGetLastError());
  k_refit<<<G, B, 0, st>>>(d_boxes, out->order, n, left.p, right.p, parent.p, flag.p, nbox.p);
  BVH_CHECK(cudaGetLastError());

  // root binary node 0 holds all n > 1 primitives
  if (n <= leaf_max) {
    BVH_CHECK(cudaStreamSynchronize(st));
    out->root = make_leaf(0, n);
    return cudaSuccess;
  }

  // SAH costs of every binary node (bottom-up), when the collapse uses them
  const bool use_sah = sah_cost != nullptr;
  DevMem<float> sahS(use_sah ? (int64_t)nb * width : 0);
  DevMem<uint8_t> sahD(use_sah ? (int64_t)nb * width : 0), sahSplit(use_sah ? n - 1 : 0);
  DevMem<int32_t> flag2(use_sah ? n - 1 : 0);
  SahArgs sah{};
  if (use_sah) {
    BVH_CHECK(sahS.alloc());
    BVH_CHECK(sahD.alloc());
    BVH_CHECK(sahSplit.alloc());
    BVH_CHECK(flag2.alloc());
    BVH_CHECK(cudaMemsetAsync(flag2.p, 0, sizeof(int32_t) * (n - 1), st));
    sah = SahArgs{left.p, right.p, parent.p, first.p, last.p, nbox.p, n, leaf_max, width,
                  (float)sah_cost->node, (float)sah_cost->prim, sahS.p, sahD.p, sahSplit.p,
                  flag2.p};
    k_sah<<<G, B, 0, st>>>(sah);
    BVH_CHECK(cudaGetLastError());
  }

  // collapse, level by level
  const int32_t cap = n;  // inner wide nodes < n
  const int64_t recs = (int64_t)cap * (width / kWidth);
  BVH_CHECK(cudaMalloc(&out->n32, sizeof(Node32) * recs));
  BVH_CHECK(cudaMalloc(&out->n64, sizeof(Node64) * recs));
  DevMem<int2> qa(cap), qb(cap);
  DevMem<int32_t> counters(2);  // [0] node counter, [1] out count
  BVH_CHECK(qa.alloc());
  BVH_CHECK(qb.alloc());
  BVH_CHECK(counters.alloc());
  int2 root_item = make_int2(0, 0);
  int32_t hc[2] = {1, 0};
  BVH_CHECK(cudaMemcpyAsync(qa.p, &root_item, sizeof root_item, cudaMemcpyHostToDevice, st));
  BVH_CHECK(cudaMemcpyAsync(counters.p, hc, sizeof hc, cudaMemcpyHostToDevice, st));
  CollapseArgs A{left.p, right.p, first.p, last.p, nbox.p, n, leaf_max,
                 out->n32, out->n64, counters.p, counters.p + 1};
  int32_t n_in = 1;
  int depth = 0;
  int2* qin = qa.p;
  int2* qout = qb.p;
  while (n_in > 0) {
    BVH_CHECK(cudaMemsetAsync(counters.p + 1, 0, sizeof(int32_t), st));
    if (width == 8)
      k_collapse<8><<<(n_in + 127) / 128, 128, 0, st>>>(A, qin, n_in, qout, sah, use_sah ? 1 : 0);
    else
      k_collapse<4><<<(n_in + 127) / 128, 128, 0, st>>>(A, qin, n_in, qout, sah, use_sah ? 1 : 0);
    BVH_CHECK(cudaGetLastError());
    BVH_CHECK(cudaMemcpyAsync(hc, counters.p, sizeof hc, cudaMemcpyDeviceToHost, st));
    BVH_CHECK(cudaStreamSynchronize(st));
    ++depth;
    n_in = hc[1];
    int2* t = qin;
    qin = qout;
    qout = t;
    if (depth > 4 * 64 + 64) return cudaErrorUnknown;  // cannot happen for < 2^31 prims
  }
  out->n_nodes = hc[0];
  out->depth = depth;
  out->root = 0;
  return cudaSuccess;
}

}  // namespace xdgcu
