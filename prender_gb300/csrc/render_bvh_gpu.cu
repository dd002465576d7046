// GPU build of the render path's binary binned-SAH tree (see render_bvh.h).
//
// Breadth first: one launch per tree level, one warp per node of the level.
// A warp bounds its node's triangles and their centroids (shuffle
// reductions), bins them along each axis into shared memory (16 bins of
// box + count per axis, float min / max as order-preserving integer
// atomics), evaluates the split candidates in the host builder's order with
// the host builder's float operations (explicitly rounded, no contraction),
// and either ends the node as a leaf or partitions its triangle range stably
// into the next level's buffer and appends its two children to the next
// level.  The host reads one counter per level.  The same tree as the host
// build (render_bvh.cpp), in milliseconds instead of hundreds of them.
#include <cuda_runtime.h>

#include <vector>

#include "render_bvh.h"

namespace pr {
namespace {

constexpr int kBins = 16;
constexpr int kMaxLeaf = 3;
constexpr float kCostNode = 3.0f;
constexpr int kWarpsPerBlock = 4;
constexpr int kBinInts = 3 * kBins * 7;  // per axis and bin: min xyz, max xyz (ordered ints), count

// float <-> int with the same order (for atomicMin / atomicMax)
__device__ __forceinline__ int ford(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float iord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

struct DBox {
  float mn[3], mx[3];
};

// Box::area of the host builder: 2 (dx dy + dy dz + dz dx), 0 when empty
__device__ __forceinline__ float box_area(const DBox& b) {
  if (b.mn[0] > b.mx[0]) return 0.0f;
  const float dx = __fsub_rn(b.mx[0], b.mn[0]), dy = __fsub_rn(b.mx[1], b.mn[1]), dz = __fsub_rn(b.mx[2], b.mn[2]);
  return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx)));
}

__device__ __forceinline__ void box_grow(DBox& a, const DBox& b) {
  for (int k = 0; k < 3; k++) {
    a.mn[k] = fminf(a.mn[k], b.mn[k]);
    a.mx[k] = fmaxf(a.mx[k], b.mx[k]);
  }
}

__device__ __forceinline__ DBox box_empty() {
  DBox b;
  for (int k = 0; k < 3; k++) {
    b.mn[k] = 3.0e38f;
    b.mx[k] = -3.0e38f;
  }
  return b;
}

// per-triangle box and centroid (the host builder's Tri)
__global__ void tri_prep(const float* __restrict__ V, const int32_t* __restrict__ F, int n, float4* __restrict__ lo,
                         float4* __restrict__ hi, float4* __restrict__ cen) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int k = 0; k < 3; k++) {
    const float* v = V + 3 * (size_t)F[3 * (size_t)t + k];
    for (int a = 0; a < 3; a++) {
      mn[a] = fminf(mn[a], v[a]);
      mx[a] = fmaxf(mx[a], v[a]);
    }
  }
  lo[t] = make_float4(mn[0], mn[1], mn[2], 0.0f);
  hi[t] = make_float4(mx[0], mx[1], mx[2], 0.0f);
  cen[t] = make_float4(__fmul_rn(0.5f, __fadd_rn(mn[0], mx[0])), __fmul_rn(0.5f, __fadd_rn(mn[1], mx[1])),
                       __fmul_rn(0.5f, __fadd_rn(mn[2], mx[2])), 0.0f);
}

// the host builder's bin index (kept in [0, kBins) for any input)
__device__ __forceinline__ int bin_of(float c, float cmn, float k) {
  return max(0, min(kBins - 1, (int)__fmul_rn(__fsub_rn(c, cmn), k)));
}

struct LevelArgs {
  const float4* lo;
  const float4* hi;
  const float4* cen;
  const int32_t* in;     // this level's triangle order
  int32_t* out;          // the next level's
  int32_t* final_order;  // leaves' triangles, where they end
  BinNode* nodes;
  const int32_t* act;    // nodes of this level
  int32_t n_act;
  int32_t* next_act;
  unsigned int* next_count;
  unsigned int* node_count;
};

__global__ void __launch_bounds__(32 * kWarpsPerBlock) split_level(LevelArgs A) {
  __shared__ int bins_all[kWarpsPerBlock][kBinInts];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int w = blockIdx.x * kWarpsPerBlock + wib;
  if (w >= A.n_act) return;  // whole warps leave together
  int* bins = bins_all[wib];
  const int id = A.act[w];
  const int first = A.nodes[id].first, count = A.nodes[id].count;
  // node box and centroid bounds
  DBox box = box_empty(), cb = box_empty();
  for (int p = first + lane; p < first + count; p += 32) {
    const int t = A.in[p];
    const float4 l = A.lo[t], h = A.hi[t], c = A.cen[t];
    box.mn[0] = fminf(box.mn[0], l.x); box.mn[1] = fminf(box.mn[1], l.y); box.mn[2] = fminf(box.mn[2], l.z);
    box.mx[0] = fmaxf(box.mx[0], h.x); box.mx[1] = fmaxf(box.mx[1], h.y); box.mx[2] = fmaxf(box.mx[2], h.z);
    cb.mn[0] = fminf(cb.mn[0], c.x); cb.mn[1] = fminf(cb.mn[1], c.y); cb.mn[2] = fminf(cb.mn[2], c.z);
    cb.mx[0] = fmaxf(cb.mx[0], c.x); cb.mx[1] = fmaxf(cb.mx[1], c.y); cb.mx[2] = fmaxf(cb.mx[2], c.z);
  }
  for (int off = 16; off > 0; off >>= 1)
    for (int k = 0; k < 3; k++) {
      box.mn[k] = fminf(box.mn[k], __shfl_xor_sync(0xffffffffu, box.mn[k], off));
      box.mx[k] = fmaxf(box.mx[k], __shfl_xor_sync(0xffffffffu, box.mx[k], off));
      cb.mn[k] = fminf(cb.mn[k], __shfl_xor_sync(0xffffffffu, cb.mn[k], off));
      cb.mx[k] = fmaxf(cb.mx[k], __shfl_xor_sync(0xffffffffu, cb.mx[k], off));
    }
  if (lane == 0)
    for (int k = 0; k < 3; k++) {
      A.nodes[id].mn[k] = box.mn[k];
      A.nodes[id].mx[k] = box.mx[k];
    }
  // bins along every axis with a centroid extent
  float kk[3];
  bool use[3];
  for (int a = 0; a < 3; a++) {
    const float ext = __fsub_rn(cb.mx[a], cb.mn[a]);
    use[a] = count > 1 && ext > 0.0f;
    kk[a] = use[a] ? __fdiv_rn(kBins * (1.0f - 1.0e-6f), ext) : 0.0f;
  }
  for (int i = lane; i < kBinInts; i += 32) {
    const int f = i % 7;
    bins[i] = f < 3 ? ford(3.0e38f) : f < 6 ? ford(-3.0e38f) : 0;
  }
  __syncwarp();
  if (count > 1) {
    for (int p = first + lane; p < first + count; p += 32) {
      const int t = A.in[p];
      const float4 l = A.lo[t], h = A.hi[t], c = A.cen[t];
      const float cc[3] = {c.x, c.y, c.z};
      for (int a = 0; a < 3; a++) {
        if (!use[a]) continue;
        int* q = bins + (a * kBins + bin_of(cc[a], cb.mn[a], kk[a])) * 7;
        atomicMin(q + 0, ford(l.x)); atomicMin(q + 1, ford(l.y)); atomicMin(q + 2, ford(l.z));
        atomicMax(q + 3, ford(h.x)); atomicMax(q + 4, ford(h.y)); atomicMax(q + 5, ford(h.z));
        atomicAdd(q + 6, 1);
      }
    }
  }
  __syncwarp();
  // split candidates of axis 'lane' (lanes 0-2), in the host builder's order
  float best = 3.0e38f;
  int best_bin = -1;
  if (lane < 3 && use[lane]) {
    const int a = lane;
    float rarea[kBins];
    int rcount[kBins];
    DBox acc = box_empty();
    int n = 0;
    for (int b = kBins - 1; b > 0; b--) {
      const int* q = bins + (a * kBins + b) * 7;
      DBox bb;
      for (int k = 0; k < 3; k++) {
        bb.mn[k] = iord(q[k]);
        bb.mx[k] = iord(q[3 + k]);
      }
      box_grow(acc, bb);
      n += q[6];
      rarea[b] = box_area(acc);
      rcount[b] = n;
    }
    DBox lacc = box_empty();
    int ln = 0;
    for (int b = 0; b < kBins - 1; b++) {
      const int* q = bins + (a * kBins + b) * 7;
      DBox bb;
      for (int k = 0; k < 3; k++) {
        bb.mn[k] = iord(q[k]);
        bb.mx[k] = iord(q[3 + k]);
      }
      box_grow(lacc, bb);
      ln += q[6];
      if (ln == 0 || rcount[b + 1] == 0) continue;
      const float cst = __fadd_rn(__fmul_rn(box_area(lacc), (float)ln), __fmul_rn(rarea[b + 1], (float)rcount[b + 1]));
      if (cst < best) {
        best = cst;
        best_bin = b;
      }
    }
  }
  // the first best over axes 0, 1, 2 (strict '<', as the host loops)
  int axis = -1, split_bin = -1;
  float bestc = 3.0e38f;
  for (int a = 0; a < 3; a++) {
    const float ca = __shfl_sync(0xffffffffu, best, a);
    const int ba = __shfl_sync(0xffffffffu, best_bin, a);
    if (ba >= 0 && ca < bestc) {
      bestc = ca;
      axis = a;
      split_bin = ba;
    }
  }
  const float area = box_area(box);
  const float split_cost = axis >= 0 && area > 0.0f ? __fadd_rn(kCostNode, __fdiv_rn(bestc, area)) : 3.0e38f;
  if (count == 1 || (count <= kMaxLeaf && (float)count <= split_cost)) {
    for (int p = first + lane; p < first + count; p += 32) A.final_order[p] = A.in[p];
    if (lane == 0) {
      A.nodes[id].left = -1;
      A.nodes[id].right = -1;
    }
    return;
  }
  // left count: the chosen bins, or half of the range when every centroid coincides
  int n_left;
  if (axis >= 0) {
    n_left = 0;
    for (int b = 0; b <= split_bin; b++) n_left += bins[(axis * kBins + b) * 7 + 6];
  } else {
    n_left = count / 2;
  }
  // stable partition of the range into the next level's order
  int lbase = 0, rbase = 0;
  for (int p0 = first; p0 < first + count; p0 += 32) {
    const int p = p0 + lane;
    const bool valid = p < first + count;
    int t = 0;
    bool left = false;
    if (valid) {
      t = A.in[p];
      if (axis >= 0) {
        const float4 c = A.cen[t];
        const float cc = axis == 0 ? c.x : axis == 1 ? c.y : c.z;
        left = bin_of(cc, cb.mn[axis], kk[axis]) <= split_bin;
      } else {
        left = (p - first) < n_left;
      }
    }
    const unsigned int lm = __ballot_sync(0xffffffffu, valid && left);
    const unsigned int rm = __ballot_sync(0xffffffffu, valid && !left);
    const unsigned int below = (1u << lane) - 1u;
    if (valid) {
      const int dst = left ? first + lbase + __popc(lm & below) : first + n_left + rbase + __popc(rm & below);
      A.out[dst] = t;
    }
    lbase += __popc(lm);
    rbase += __popc(rm);
  }
  if (lane == 0) {
    const int c0 = (int)atomicAdd(A.node_count, 2u);
    A.nodes[id].left = c0;
    A.nodes[id].right = c0 + 1;
    A.nodes[c0].first = first;
    A.nodes[c0].count = n_left;
    A.nodes[c0 + 1].first = first + n_left;
    A.nodes[c0 + 1].count = count - n_left;
    const int q = (int)atomicAdd(A.next_count, 2u);
    A.next_act[q] = c0;
    A.next_act[q + 1] = c0 + 1;
  }
}

__global__ void iota(int32_t* a, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = i;
}

}  // namespace

cudaError_t build_render_bvh_binary_gpu(const float* vertices, int32_t n_vertices, const int32_t* faces,
                                        int32_t n_faces, cudaStream_t s, std::vector<BinNode>& tree,
                                        std::vector<int32_t>& order) {
  if (n_faces <= 0 || n_vertices <= 0) return cudaErrorInvalidValue;
  const size_t n = (size_t)n_faces, max_nodes = 2 * n;
  // one allocation for every work array
  const size_t bytes_v = sizeof(float) * 3 * (size_t)n_vertices, bytes_f = sizeof(int32_t) * 3 * n;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t off_f = al(bytes_v), off_lo = off_f + al(bytes_f), off_hi = off_lo + al(16 * n),
               off_c = off_hi + al(16 * n), off_i0 = off_c + al(16 * n), off_i1 = off_i0 + al(4 * n),
               off_fin = off_i1 + al(4 * n), off_nodes = off_fin + al(4 * n),
               off_a0 = off_nodes + al(sizeof(BinNode) * max_nodes), off_a1 = off_a0 + al(4 * n),
               off_cnt = off_a1 + al(4 * n), total = off_cnt + 256;
  unsigned char* base = nullptr;
  cudaError_t e = cudaMalloc(&base, total);
  if (e != cudaSuccess) return e;
  float* dV = (float*)base;
  int32_t* dF = (int32_t*)(base + off_f);
  float4* lo = (float4*)(base + off_lo);
  float4* hi = (float4*)(base + off_hi);
  float4* cen = (float4*)(base + off_c);
  int32_t* buf[2] = {(int32_t*)(base + off_i0), (int32_t*)(base + off_i1)};
  int32_t* fin = (int32_t*)(base + off_fin);
  BinNode* nodes = (BinNode*)(base + off_nodes);
  int32_t* act[2] = {(int32_t*)(base + off_a0), (int32_t*)(base + off_a1)};
  unsigned int* cnt = (unsigned int*)(base + off_cnt);  // [0] nodes, [1] next level
  unsigned int hcnt[2] = {1u, 0u};
  int32_t h_act0 = 0;
  BinNode root{};
  root.first = 0;
  root.count = n_faces;
  root.left = root.right = -1;
  unsigned int n_act = 1, level = 0;
  e = cudaMemcpyAsync(dV, vertices, bytes_v, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dF, faces, bytes_f, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(nodes, &root, sizeof(root), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(act[0], &h_act0, sizeof(h_act0), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, hcnt, sizeof(hcnt), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    tri_prep<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dV, dF, n_faces, lo, hi, cen);
    iota<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(buf[0], n_faces);
    e = cudaGetLastError();
  }
  // a binary tree over n triangles with at least one per leaf is at most n levels deep
  while (e == cudaSuccess && n_act > 0) {
    if (level > (unsigned)n_faces) {
      e = cudaErrorUnknown;
      break;
    }
    e = cudaMemsetAsync(cnt + 1, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) break;
    LevelArgs A;
    A.lo = lo;
    A.hi = hi;
    A.cen = cen;
    A.in = buf[level & 1];
    A.out = buf[(level + 1) & 1];
    A.final_order = fin;
    A.nodes = nodes;
    A.act = act[level & 1];
    A.n_act = (int32_t)n_act;
    A.next_act = act[(level + 1) & 1];
    A.next_count = cnt + 1;
    A.node_count = cnt;
    split_level<<<(n_act + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, 0, s>>>(A);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hcnt, cnt, sizeof(hcnt), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    n_act = hcnt[1];
    level++;
  }
  if (e == cudaSuccess) {
    tree.resize(hcnt[0]);
    order.resize(n);
    e = cudaMemcpyAsync(tree.data(), nodes, sizeof(BinNode) * hcnt[0], cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(order.data(), fin, 4 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  cudaFree(base);
  return e;
}

}  // namespace pr
