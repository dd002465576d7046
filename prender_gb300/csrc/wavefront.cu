// Wavefront renderer: the same estimator as the megakernel (path_logic.cuh),
// scheduled as a loop of small kernels over a pool of P path slots held in
// HBM as structure-of-arrays:
//
//   wf_shade    one thread per slot: shade the last hit of a live path
//               (queue its shadow rays and its next segment, or end it), or
//               refill a free slot -- first with a glass branch waiting in
//               the spawn ring, else with the next camera sample
//   wf_extend   closest hit for every queued segment (compacted queue)
//   wf_shadow   any hit for every queued shadow ray (compacted queue)
//   wf_control  one thread: swap the per-iteration counters and decide
//               whether another iteration is needed
//
// The loop runs on the device: the four kernels are the body of a CUDA-graph
// 'while' node whose condition wf_control sets, so a whole frame is one
// graph launch with no host round trips.  Paths of very uneven length
// (glass, media, roulette) no longer hold a warp hostage: every launch works
// on compacted queues of identical work.
//
// Accumulation is in 64-bit fixed point: a path adds its radiance to its
// camera sample's slot (only samples whose glass split into branches need
// the slot), the last branch to finish applies the per-sample weight and
// luminance clamp (render.h:1353-1384) and adds the sample to its pixel.
// Integer sums are associative, so the image does not depend on the order
// in which paths finish.
#include <cuda_runtime.h>

#include "path_logic.cuh"
#include "wavefront.h"

namespace pr {

__constant__ DevScene c_scene;
__constant__ RenderCfg c_cfg;
__constant__ WfBufs c_buf;

constexpr float kSampleScale = 4294967296.0f;        // 2^32
constexpr double kSampleInv = 1.0 / 4294967296.0;
constexpr double kPixelScale = 1099511627776.0;      // 2^40
constexpr double kPixelInv = 1.0 / 1099511627776.0;

enum : int { SLOT_FREE = 0, SLOT_RAY = 1, SLOT_HIT = 2 };

__device__ __forceinline__ void store_state(const WfBufs& B, int i, const PathState& ps, int slot_state) {
  B.o[i] = make_float4(ps.o.x, ps.o.y, ps.o.z, __int_as_float(ps.depth));
  B.d[i] = make_float4(ps.d.x, ps.d.y, ps.d.z, __int_as_float(ps.dp | (slot_state << 1)));
  B.beta[i] = make_float4(ps.beta.x, ps.beta.y, ps.beta.z, __uint_as_float(ps.branch));
  B.dpw[i] = make_float4(ps.dpw.x, ps.dpw.y, ps.dpw.z, __uint_as_float(ps.draws));
  B.L[i] = make_float4(ps.L.x, ps.L.y, ps.L.z, 0.0f);
}

__device__ __forceinline__ void load_state(const WfBufs& B, int i, PathState& ps) {
  const float4 o = B.o[i], d = B.d[i], b = B.beta[i], w = B.dpw[i], l = B.L[i];
  ps.o = f3(o.x, o.y, o.z);
  ps.depth = __float_as_int(o.w);
  ps.d = f3(d.x, d.y, d.z);
  ps.dp = __float_as_int(d.w) & 1;
  ps.beta = f3(b.x, b.y, b.z);
  ps.branch = __float_as_uint(b.w);
  ps.dpw = f3(w.x, w.y, w.z);
  ps.draws = __float_as_uint(w.w);
  ps.L = f3(l.x, l.y, l.z);
}

// warp-aggregated append to a counter; returns this lane's slot
__device__ __forceinline__ unsigned int append(unsigned int* counter, bool want) {
  const unsigned int mask = __ballot_sync(__activemask(), want);
  if (!want) return 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  unsigned int base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned int)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  return base + (unsigned int)__popc(mask & ((1u << lane) - 1u));
}

// warp-aggregated append of n entries per lane (contiguous per lane, in
// lane order); returns this lane's first slot
__device__ __forceinline__ unsigned int append_n(unsigned int* counter, unsigned int n) {
  const unsigned int active = __activemask();
  if (active != 0xffffffffu) return n ? atomicAdd(counter, n) : 0u;  // partial warp: one atomic per lane
  const int lane = threadIdx.x & 31;
  unsigned int incl = n;  // inclusive prefix sum over lanes 0..lane
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned int v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += v;
  }
  const unsigned int total = __shfl_sync(0xffffffffu, incl, 31);
  unsigned int base = 0;
  if (lane == 0 && total) base = atomicAdd(counter, total);
  base = __shfl_sync(0xffffffffu, base, 0);
  return base + incl - n;
}

__device__ __forceinline__ void pixel_of(const RenderCfg& cfg, uint64_t g, int& x, int& y, uint64_t& kg) {
  const uint64_t wh = (uint64_t)cfg.width * cfg.height;
  const uint64_t k = g / wh;
  const uint32_t pix = (uint32_t)(g - k * wh);
  x = (int)(pix % (uint32_t)cfg.width);
  y = (int)(pix / (uint32_t)cfg.width);
  kg = cfg.sample_offset + c_buf.pass_first + k;
}

__device__ void add_to_pixel(const WfBufs& B, const RenderCfg& cfg, uint64_t g, float3 L) {
  int x, y;
  uint64_t kg;
  pixel_of(cfg, g, x, y, kg);
  const float3 v = finish_sample(cfg, L, B.err);
  long long* px = B.pix + 3 * ((size_t)(cfg.height - y - 1) * cfg.width + x);
  atomicAdd(reinterpret_cast<unsigned long long*>(px + 0), (unsigned long long)llrint((double)v.x * kPixelScale));
  atomicAdd(reinterpret_cast<unsigned long long*>(px + 1), (unsigned long long)llrint((double)v.y * kPixelScale));
  atomicAdd(reinterpret_cast<unsigned long long*>(px + 2), (unsigned long long)llrint((double)v.z * kPixelScale));
}

// a branch is done: a sample that never split finishes at once; otherwise
// the branch adds to the sample slot and the last one finishes the sample
__device__ void end_path(const WfBufs& B, const RenderCfg& cfg, const PathState& ps, uint64_t g) {
  if (ps.branch == 0) {
    add_to_pixel(B, cfg, g, ps.L);
    return;
  }
  long long* s = B.samp + 3 * g;
  atomicAdd(reinterpret_cast<unsigned long long*>(s + 0), (unsigned long long)__float2ll_rn(ps.L.x * kSampleScale));
  atomicAdd(reinterpret_cast<unsigned long long*>(s + 1), (unsigned long long)__float2ll_rn(ps.L.y * kSampleScale));
  atomicAdd(reinterpret_cast<unsigned long long*>(s + 2), (unsigned long long)__float2ll_rn(ps.L.z * kSampleScale));
  __threadfence();
  if (atomicSub(B.live + g, 1) == 1) {
    __threadfence();
    const volatile long long* vs = s;
    const float3 L = f3((float)((double)vs[0] * kSampleInv), (float)((double)vs[1] * kSampleInv),
                        (float)((double)vs[2] * kSampleInv));
    add_to_pixel(B, cfg, g, L);
  }
}

// ---- subsurface frames of the wavefront form -------------------------------
// The plain form keeps a sample's frames in registers (render.cu); here the
// branches of one camera sample run in different slots at the same time, so
// the frames live in the pool: fixed-point sums (the cut decision then does
// not depend on the order in which branches end) and a count of open
// branches and inner frames, the last of which closes the frame.

__device__ __forceinline__ void fx_add3(long long* p, float3 v) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p + 0), (unsigned long long)__float2ll_rn(v.x * kSampleScale));
  atomicAdd(reinterpret_cast<unsigned long long*>(p + 1), (unsigned long long)__float2ll_rn(v.y * kSampleScale));
  atomicAdd(reinterpret_cast<unsigned long long*>(p + 2), (unsigned long long)__float2ll_rn(v.z * kSampleScale));
}

__device__ __forceinline__ float3 fx_read3(const long long* p) {
  const volatile long long* v = p;
  return f3((float)((double)v[0] * kSampleInv), (float)((double)v[1] * kSampleInv), (float)((double)v[2] * kSampleInv));
}

// radiance x of a branch (or of a closing frame) goes to frame f, or to the camera sample
__device__ __forceinline__ void frame_add(const WfBufs& B, int f, uint64_t g, float3 x) {
  if (x.x == 0.0f && x.y == 0.0f && x.z == 0.0f) return;
  fx_add3(f >= 0 ? B.fr_c + 3 * (size_t)f : B.samp + 3 * g, x);
}

// a new frame inside parent with one open item (the branch that opens it)
__device__ int frame_alloc(const WfBufs& B, int parent, float3 scale, float thr, float3 e, float3 c) {
  const unsigned int f = atomicAdd(&B.ctl->frame_next, 1u);
  if (f >= B.frame_cap) {
    atomicOr(B.err, PR_DEV_QUEUE_OVERFLOW);
    return -2;
  }
  long long* pc = B.fr_c + 3 * (size_t)f;
  long long* pe = B.fr_e + 3 * (size_t)f;
  pc[0] = __float2ll_rn(c.x * kSampleScale);
  pc[1] = __float2ll_rn(c.y * kSampleScale);
  pc[2] = __float2ll_rn(c.z * kSampleScale);
  pe[0] = __float2ll_rn(e.x * kSampleScale);
  pe[1] = __float2ll_rn(e.y * kSampleScale);
  pe[2] = __float2ll_rn(e.z * kSampleScale);
  B.fr_scale[f] = make_float4(scale.x, scale.y, scale.z, thr);
  B.fr_link[f] = make_int2(parent, 1);
  return (int)f;
}

// one open item of frame f (-1: of the camera sample g) ended: close every
// frame that has nothing open left (its C + E to its parent unless
// |C / scale| exceeds its bound), and finish the sample when its last item ends
__device__ void frame_release(const WfBufs& B, const RenderCfg& cfg, int f, uint64_t g) {
  for (int level = 0; level < 64; level++) {
    __threadfence();  // this item's sums before its count
    if (f < 0) {
      if (atomicSub(B.live + g, 1) == 1) {
        __threadfence();
        add_to_pixel(B, cfg, g, fx_read3(B.samp + 3 * g));
      }
      return;
    }
    if (atomicSub(&B.fr_link[f].y, 1) != 1) return;
    __threadfence();
    const float3 c = fx_read3(B.fr_c + 3 * (size_t)f), e = fx_read3(B.fr_e + 3 * (size_t)f);
    const float4 sc = B.fr_scale[f];
    const float3 q = f3(sc.x != 0.0f ? c.x / sc.x : 0.0f, sc.y != 0.0f ? c.y / sc.y : 0.0f,
                        sc.z != 0.0f ? c.z / sc.z : 0.0f);
    const int parent = B.fr_link[f].x;
    if (!(sqrtf(dot(q, q)) > sc.w)) frame_add(B, parent, g, c + e);
    f = parent;
  }
  atomicOr(B.err, PR_DEV_LOOP_CAP);
}

__global__ void __launch_bounds__(256) wf_reset(unsigned int n_slots) {
  const WfBufs& B = c_buf;
  const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_slots) B.d[i] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(SLOT_FREE << 1));
  if (i == 0) {
    WfCtl* c = B.ctl;
    c->ext_count = 0;
    c->sh_count = 0;
    c->ext_fetch = 0;
    c->sh_fetch = 0;
    c->spawn_head = 0;
    c->spawn_tail = 0;
    c->spawn_ready = 0;
    c->next_sample = 0;
    c->iterations = 0;
    c->work = 1;
    c->head_start = 0;
    c->frame_next = 0;
  }
}

// One iteration's shading of every slot.  SSS: scenes with subsurface
// materials (the fuller shade() with the dipole and the single-scattering
// walk, and the frames above); every camera sample then ends through its
// sample slot, since frames may take radiance from any of its branches.
template <bool SSS, bool EXT>
__device__ __forceinline__ void wf_shade_impl() {
  const DevScene& S = c_scene;
  const RenderCfg& cfg = c_cfg;
  const WfBufs& B = c_buf;
  WfCtl* ctl = B.ctl;
  const unsigned int stride = gridDim.x * blockDim.x;
  const unsigned int ready = ctl->spawn_ready;  // spawns written in earlier iterations
  const unsigned int head_start = ctl->head_start;
  const bool samples_left = ctl->next_sample < B.pass_samples;
  for (unsigned int base = blockIdx.x * blockDim.x; base < B.n_slots; base += stride) {
    const unsigned int i = base + threadIdx.x;
    int state = SLOT_FREE;
    bool was_free = true;  // free before this iteration (its record already says so)
    PathState ps;
    uint64_t g = 0;
    bool has_ray = false;
    int n_shadow = 0;
    int fr = -1;      // the slot's innermost subsurface frame (SSS)
    int nee_to = -1;  // where this vertex's shadow terms go (SSS: a frame's E, or the path)
    if (i < B.n_slots) {
      state = __float_as_int(B.d[i].w) >> 1;
      was_free = state == SLOT_FREE;
      if (state == SLOT_HIT) {
        load_state(B, i, ps);
        g = B.sample[i];
        // shadow rays of the previous vertex that were not blocked
        float3 nee = f3(0, 0, 0);
        for (int k = 0; k < 3; k++) {
          const float4 c = B.nee[3 * i + k];
          nee += f3(c.x, c.y, c.z);
        }
        if (SSS) {
          fr = __float_as_int(B.L[i].w) - 1;
          const int nf = B.neef[i];
          // the frame-opening vertex's own terms join the frame's E, outside
          // its bound (as the megakernel's F.E; the reference bounds only
          // weight * incoming, Subsurface_Scattering.h:1061-1066)
          if (nf >= 0) fx_add3(B.fr_e + 3 * (size_t)nf, nee);
          else ps.L += nee;
        } else {
          ps.L += nee;
        }
        const float4 h4 = B.hit[i];
        FastHit h;
        h.t = h4.x;
        h.ent = __float_as_int(h4.y);
        h.slot = __float_as_int(h4.z);
        h.u = h4.w;
        h.v = B.hitv[i];
        int kg_x, kg_y;
        uint64_t kg;
        pixel_of(cfg, g, kg_x, kg_y, kg);
        const uint64_t sample_id = kg * (uint64_t)cfg.width * (uint64_t)cfg.height + (uint64_t)kg_y * cfg.width + kg_x;
        ShadowReq sh[3];
        int nsh = 0;
        PathState child;
        int r;
        if (SSS) {
          const float3 Lb = ps.L;
          SssFrameOut fo;
          fo.open = 0;
          r = shade<true, true, true>(S, cfg, ps, h.ent >= 0, h, sample_id, sh, nsh, child, B.err, nullptr,
                                      nullptr, nullptr, &fo);
          if (fo.open) {
            // the branch moves into a new frame (or two nested ones): what it
            // gathered before this vertex belongs outside, the vertex's own
            // terms to the frame, its continuation inside (render.cu does the same)
            frame_add(B, fr, g, Lb);
            const int f = frame_alloc(B, fr, fo.scale, fo.thr, ps.L - Lb, fo.open == 1 ? fo.inner : f3(0, 0, 0));
            int in = f;
            if (f >= 0 && fo.open == 2) in = frame_alloc(B, f, fo.scale2, fo.thr2, f3(0, 0, 0), fo.inner);
            if (f >= 0 && in >= 0) {
              nee_to = fo.nee_inner ? -1 : f;
              ps.L = f3(0, 0, 0);
              fr = in;
            } else {
              r = SHADE_END;  // frames exhausted (reported): the branch ends
              nsh = 0;
            }
          }
          if (r == SHADE_END && nsh > 0) {  // shadow terms are only queued for continuing paths
            atomicOr(B.err, PR_DEV_BAD_INDEX);
            nsh = 0;
          }
        } else {
          r = shade<false, true, EXT>(S, cfg, ps, h.ent >= 0, h, sample_id, sh, nsh, child, B.err);
        }
        for (int k = 0; k < 3; k++) {
          if (k < nsh) {
            B.nee[3 * i + k] = make_float4(sh[k].contrib.x, sh[k].contrib.y, sh[k].contrib.z, 0.0f);
            B.sh_o[3 * i + k] = make_float4(sh[k].o.x, sh[k].o.y, sh[k].o.z, sh[k].tmax);
            B.sh_d[3 * i + k] = make_float4(sh[k].d.x, sh[k].d.y, sh[k].d.z, 0.0f);
          } else {
            B.nee[3 * i + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          }
        }
        if (r == SHADE_SPLIT) {
          if (SSS && fr >= 0) atomicAdd(&B.fr_link[fr].y, 1);
          else atomicAdd(B.live + g, 1);
          const unsigned int t = atomicAdd(&ctl->spawn_tail, 1u);
          // entries from head_start on may still be unread this iteration
          if (t - head_start >= B.spawn_cap) {
            atomicOr(B.err, PR_DEV_QUEUE_OVERFLOW);
          } else {
            const unsigned int q = t % B.spawn_cap;
            B.sp_o[q] = make_float4(child.o.x, child.o.y, child.o.z, __int_as_float(child.depth));
            B.sp_d[q] = make_float4(child.d.x, child.d.y, child.d.z, __int_as_float(child.dp));
            B.sp_beta[q] = make_float4(child.beta.x, child.beta.y, child.beta.z, __uint_as_float(child.branch));
            B.sp_dpw[q] = make_float4(child.dpw.x, child.dpw.y, child.dpw.z, __uint_as_float(child.draws));
            B.sp_sample[q] = g;
            if (SSS) B.sp_frame[q] = fr;
          }
        }
        if (r == SHADE_END) {
          if (SSS) {
            frame_add(B, fr, g, ps.L);
            frame_release(B, cfg, fr, g);
          } else {
            end_path(B, cfg, ps, g);
          }
          state = SLOT_FREE;
        } else {
          has_ray = true;
        }
        n_shadow = nsh;
      }
      if (state == SLOT_FREE) {
        // refill: a waiting glass branch first, else the next camera sample
        const unsigned int t = (head_start < ready) ? atomicAdd(&ctl->spawn_head, 1u) : ready;
        if (t < ready) {
          const unsigned int q = t % B.spawn_cap;
          const float4 o = B.sp_o[q], d = B.sp_d[q], b = B.sp_beta[q], w = B.sp_dpw[q];
          ps.o = f3(o.x, o.y, o.z);
          ps.depth = __float_as_int(o.w);
          ps.d = f3(d.x, d.y, d.z);
          ps.dp = __float_as_int(d.w);
          ps.beta = f3(b.x, b.y, b.z);
          ps.branch = __float_as_uint(b.w);
          ps.dpw = f3(w.x, w.y, w.z);
          ps.draws = __float_as_uint(w.w);
          ps.L = f3(0, 0, 0);
          g = B.sp_sample[q];
          if (SSS) fr = B.sp_frame[q];
          has_ray = true;
        } else if (samples_left) {
          const unsigned long long s = atomicAdd(&ctl->next_sample, 1ull);
          if (s < B.pass_samples) {
            g = s;
            int x, y;
            uint64_t kg;
            pixel_of(cfg, g, x, y, kg);
            float3 o, d;
            camera_ray(cfg, x, y, kg, o, d);
            root_path(ps, o, d);
            B.live[g] = 1;
            fr = -1;
            has_ray = true;
          }
        }
      }
      if (has_ray) {
        store_state(B, i, ps, SLOT_RAY);
        B.sample[i] = g;
        if (SSS) {
          B.L[i].w = __int_as_float(fr + 1);
          B.neef[i] = nee_to;
        }
      } else if (!was_free) {  // its path ended and nothing refilled it
        B.d[i] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(SLOT_FREE << 1));
      }
    }
    const unsigned int q = append(&ctl->ext_count, has_ray);
    if (has_ray) B.extq[q] = i;
    // shadow rays: a lane's (up to three) rays share origin and light, so
    // they go to adjacent queue entries and trace side by side in a warp
    const unsigned int qs = append_n(&ctl->sh_count, (unsigned int)n_shadow);
    for (int k = 0; k < n_shadow; k++) B.shq[qs + k] = 3 * i + k;
  }
}

// 6 blocks of 128 per SM (80 registers, a few spilled): measured on GB300
// over 4 / 5 / 6 / 7 / 8 / 10 blocks, mesh Cornell box 1024x768x64 spp,
// wf_shade 108 / 99 / 94 / 96 / 102 / 110 ms per frame
__global__ void __launch_bounds__(128, 6) wf_shade() { wf_shade_impl<false, false>(); }
// scenes with parallel, spot or infinity lights, textures or IBL images
__global__ void __launch_bounds__(128, 4) wf_shade_ext() { wf_shade_impl<false, true>(); }
// scenes with subsurface materials (any light kind)
__global__ void __launch_bounds__(128, 3) wf_shade_sss() { wf_shade_impl<true, true>(); }

// Persistent traversal with ray replacement (Aila & Laine 2009, "Understanding
// the efficiency of ray traversal on GPUs", dynamic ray fetch): the lanes of a
// warp advance their rays one step at a time (the non-mesh entities of the
// list in one step, then one mesh node with its leaves per step) and, once
// half of the warp holds no ray, take the next queue entries with one
// warp-aggregated atomic (half: measured on GB300 over 4 / 8 / 16 / 32 idle
// lanes, mesh Cornell box 1024x768x64 spp: 98 / 109 / 112 / 99 Mpaths/s).  A ray visits the same nodes and triangles in the
// same order as fast_closest / fast_occluded, so the results are those of the
// per-ray loop; only the schedule changes: a lane whose ray ends early no
// longer idles until the longest ray of its warp is done.
constexpr int kRefillLanes = 16;
constexpr unsigned int kWarpStepCap = 1u << 26;

struct TraceLane {
  WRay ray;
  float tmax;        // current closest (closest hit) or the ray's limit (any hit)
  int ent;           // next entity of the list to test (the current mesh while in_mesh)
  int sp;            // node groups on the traversal stack
  bool in_mesh;      // inside the traversal of mesh 'ent'
  WGroup g;          // the current node group
  FastHit h;
};

__device__ __forceinline__ void lane_start(TraceLane& r, float3 o, float3 d, float tmax) {
  r.ray = make_wray(o, d);
  r.tmax = tmax;
  r.ent = 0;
  r.sp = 0;
  r.in_mesh = false;
  r.g.base = 0;
  r.g.bits = 0;
  r.h.t = tmax;
  r.h.ent = -1;
  r.h.slot = -1;
  r.h.u = r.h.v = 0.0f;
}

// one step of a ray; returns true when the ray is done (ANY: r.h.ent >= 0
// means occluded)
template <bool ANY>
__device__ __forceinline__ bool lane_step(const DevScene& S, TraceLane& r, WGroup* stack, TraceStats& st,
                                          uint32_t* err) {
  if (!r.in_mesh) {
    // non-mesh entities up to the next mesh, in list order
    while (r.ent < S.n_ents) {
      const int i = r.ent;
      const GEntF& e = S.entf[i];
      if (e.type == PR_ENT_POLYGON) {
        r.g = wgroup_root(e.node_base, r.ray.oct);
        r.sp = 0;
        r.in_mesh = true;
        break;
      }
      float t = r.tmax, rest = 0.0f;
      bool got = false;
      if (e.type == PR_ENT_SPHERE) got = fast_sphere(S.ents[i], r.ray.o, r.ray.d, r.tmax, t, rest);
      else if (e.type == PR_ENT_UVPLANE) got = fast_uvplane(e, r.ray.o, r.ray.d, r.tmax, t);
      else if (e.type == PR_ENT_CIRCLE) got = fast_circle(e, r.ray.o, r.ray.d, r.tmax, t);
      r.ent++;
      if (ANY && got) {  // the test itself keeps t below the limit
        r.h.ent = i;
        return true;
      }
      if (got && t < r.tmax) {
        r.h.ent = i;
        r.h.slot = -1;
        r.h.u = rest;  // a sphere's remainder of t (0 for planes and disks)
        r.h.v = 0.0f;
        r.tmax = t;
        r.h.t = t;
      }
    }
    return !r.in_mesh;  // past the last entity
  }
  // one node of the current mesh with its leaf triangles (fast_qbvh's loop body)
  if ((r.g.bits & 0xFFu) == 0) r.g = stack[--r.sp];  // stacked groups always hold a pending child
  const int child = wgroup_next(r.g, r.ray.oct);
  if (r.g.bits & 0xFFu) {
    if (r.sp >= kWStack) {
      atomicOr(err, PR_DEV_STACK_OVERFLOW);
      r.in_mesh = false;
      r.ent = S.n_ents;
      return true;
    }
    stack[r.sp++] = r.g;
  }
  st.nodes++;
  uint32_t tm;
  int tb;
  wnode_visit(S.rnodes + child, r.ray, r.tmax, r.g, tm, tb);
  while (tm) {
    const int k = __ffs(tm) - 1;
    tm &= tm - 1u;
    st.tris++;
    float t, uu, vv;
    if (fast_tri(S.rtris + 3 * (size_t)(tb + k), r.ray.o, r.ray.d, r.tmax, t, uu, vv)) {
      r.h.ent = r.ent;
      r.h.slot = tb + k;
      if (ANY) return true;
      r.tmax = t;
      r.h.t = t;
      r.h.u = uu;
      r.h.v = vv;
    }
  }
  if ((r.g.bits & 0xFFu) == 0 && r.sp == 0) {
    r.in_mesh = false;  // this mesh is done
    r.ent++;
    return r.ent >= S.n_ents;
  }
  return false;
}

// The persistent loop shared by wf_extend and wf_shadow.  fetch(idx, r)
// starts queue entry idx on the lane; finish(r) stores its result.
template <bool ANY, class Fetch, class Finish>
__device__ __forceinline__ void persistent_trace(const DevScene& S, unsigned int n, unsigned int* counter,
                                                 Fetch fetch, Finish finish, TraceStats& st, unsigned int& segs,
                                                 uint32_t* err) {
  const int lane = threadIdx.x & 31;
  TraceLane r;
  WGroup stack[kWStack];
  bool busy = false, exhausted = false;
  for (unsigned int step = 0;; step++) {
    const unsigned int idle = __ballot_sync(0xffffffffu, !busy && !exhausted);
    const unsigned int live = __ballot_sync(0xffffffffu, busy);
    if (idle == 0 && live == 0) break;
    if (step >= kWarpStepCap) {  // warp-uniform: every lane leaves together
      if (lane == 0) atomicOr(err, PR_DEV_LOOP_CAP);
      break;
    }
    if (idle && (__popc(idle) >= kRefillLanes || live == 0)) {
      const int leader = __ffs(idle) - 1;
      unsigned int base = 0;
      if (lane == leader) base = atomicAdd(counter, (unsigned int)__popc(idle));
      base = __shfl_sync(0xffffffffu, base, leader);
      if ((idle >> lane) & 1) {
        const unsigned int idx = base + __popc(idle & ((1u << lane) - 1u));
        if (idx < n) {
          fetch(idx, r);
          busy = true;
          segs++;
        } else {
          exhausted = true;
        }
      }
    }
    if (busy && lane_step<ANY>(S, r, stack, st, err)) {
      finish(r);
      busy = false;
    }
  }
}

__device__ __forceinline__ void add_trace_counters(const WfBufs& B, unsigned int segs, const TraceStats& st, bool shadow) {
  if (!B.counters) return;
  unsigned long long a = segs, c = st.nodes, dd = st.tris;
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, off);
    c += __shfl_down_sync(0xffffffffu, c, off);
    dd += __shfl_down_sync(0xffffffffu, dd, off);
  }
  if ((threadIdx.x & 31) == 0 && a) {
    atomicAdd(B.counters + 1, a);
    atomicAdd(B.counters + 2, c);
    atomicAdd(B.counters + 3, dd);
    if (shadow) {  // the shadow kernel's own share
      atomicAdd(B.counters + 6, a);
      atomicAdd(B.counters + 7, c);
      atomicAdd(B.counters + 8, dd);
    }
  }
}

__global__ void __launch_bounds__(128, 8) wf_extend() {
  const DevScene& S = c_scene;
  const WfBufs& B = c_buf;
  TraceStats st{0, 0};
  unsigned int segs = 0;
  int slot = 0, dflag = 0;
  persistent_trace<false>(
      S, B.ctl->ext_count, &B.ctl->ext_fetch,
      [&](unsigned int idx, TraceLane& r) {
        slot = B.extq[idx];
        const float4 o4 = B.o[slot], d4 = B.d[slot];
        dflag = __float_as_int(d4.w) & 1;
        lane_start(r, f3(o4.x, o4.y, o4.z), f3(d4.x, d4.y, d4.z), 3.0e38f);
      },
      [&](const TraceLane& r) {
        const bool hit = r.h.ent >= 0;
        B.hit[slot] = make_float4(r.h.t, __int_as_float(hit ? r.h.ent : -1), __int_as_float(r.h.slot), r.h.u);
        B.hitv[slot] = r.h.v;
        B.d[slot].w = __int_as_float(dflag | (SLOT_HIT << 1));
      },
      st, segs, B.err);
  add_trace_counters(B, segs, st, false);
}

__global__ void __launch_bounds__(128, 8) wf_shadow() {
  const DevScene& S = c_scene;
  const WfBufs& B = c_buf;
  TraceStats st{0, 0};
  unsigned int segs = 0;
  int item = 0;
  persistent_trace<true>(
      S, B.ctl->sh_count, &B.ctl->sh_fetch,
      [&](unsigned int idx, TraceLane& r) {
        item = B.shq[idx];
        const float4 o4 = B.sh_o[item], d4 = B.sh_d[item];
        lane_start(r, f3(o4.x, o4.y, o4.z), f3(d4.x, d4.y, d4.z), o4.w);
      },
      [&](const TraceLane& r) {
        if (r.h.ent >= 0) B.nee[item] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      },
      st, segs, B.err);
  add_trace_counters(B, segs, st, true);
}

__global__ void wf_control(cudaGraphConditionalHandle handle, int use_graph) {
  const WfBufs& B = c_buf;
  WfCtl* c = B.ctl;
  // tickets past the ready spawns took nothing
  if (c->spawn_head > c->spawn_ready) c->spawn_head = c->spawn_ready;
  const bool pending_spawns = c->spawn_tail > c->spawn_head;
  if (c->spawn_tail - c->spawn_head > B.spawn_cap) atomicOr(B.err, PR_DEV_QUEUE_OVERFLOW);
  c->spawn_ready = c->spawn_tail;
  c->head_start = c->spawn_head;
  const bool more_samples = c->next_sample < B.pass_samples;
  if (c->next_sample > B.pass_samples) c->next_sample = B.pass_samples;
  unsigned int work = (c->ext_count > 0 || pending_spawns || more_samples) ? 1u : 0u;
  c->iterations++;
  if (c->iterations >= B.max_iterations) {
    atomicOr(B.err, PR_DEV_LOOP_CAP);
    work = 0;
  }
  if (B.counters) {
    B.counters[4] += c->ext_count;
    B.counters[5] += 1;  // iterations
  }
  c->ext_count = 0;
  c->sh_count = 0;
  c->ext_fetch = 0;
  c->sh_fetch = 0;
  c->work = work;
  if (use_graph) cudaGraphSetConditional(handle, work);
}

// fixed-point pixel sums -> float image (reference row order), times the
// sensor response (render.h:1405-1409); accumulate adds to the output
__global__ void wf_resolve(float* __restrict__ out, int n3, int accumulate, float sensor) {
  const WfBufs& B = c_buf;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  const float v = (float)((double)B.pix[i] * kPixelInv) * sensor;
  out[i] = accumulate ? out[i] + v : v;
}

// ------------------------------------------------------------------ host
cudaError_t wf_set_constants(const DevScene& S, const RenderCfg& cfg, const WfBufs& B, cudaStream_t s) {
  cudaError_t e = cudaMemcpyToSymbolAsync(c_scene, &S, sizeof(DevScene), 0, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_cfg, &cfg, sizeof(RenderCfg), 0, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_buf, &B, sizeof(WfBufs), 0, cudaMemcpyHostToDevice, s);
  return e;
}

static void launch_shade(const WfLaunch& L, cudaStream_t s) {
  if (L.sss) wf_shade_sss<<<L.shade_blocks, 128, 0, s>>>();
  else if (L.ext) wf_shade_ext<<<L.shade_blocks, 128, 0, s>>>();
  else wf_shade<<<L.shade_blocks, 128, 0, s>>>();
}

static void launch_body(const WfLaunch& L, cudaGraphConditionalHandle handle, int use_graph, cudaStream_t s) {
  launch_shade(L, s);
  wf_extend<<<L.trace_blocks, 128, 0, s>>>();
  wf_shadow<<<L.trace_blocks, 128, 0, s>>>();
  wf_control<<<1, 1, 0, s>>>(handle, use_graph);
}

cudaError_t wf_reset_launch(unsigned int n_slots, cudaStream_t s) {
  wf_reset<<<(n_slots + 255) / 256, 256, 0, s>>>(n_slots);
  return cudaGetLastError();
}

// builds the graph  [while work { shade; extend; shadow; control }]
cudaError_t wf_build_graph(const WfLaunch& L, cudaStream_t s, cudaGraphExec_t* exec) {
  cudaGraph_t graph;
  cudaError_t e = cudaGraphCreate(&graph, 0);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle handle;
  e = cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) { cudaGraphDestroy(graph); return e; }
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = handle;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &p);
  if (e != cudaSuccess) { cudaGraphDestroy(graph); return e; }
  cudaGraph_t body = p.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) { cudaGraphDestroy(graph); return e; }
  launch_body(L, handle, 1, s);
  cudaError_t e2 = cudaGetLastError();
  e = cudaStreamEndCapture(s, &body);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  return e;
}

// host-driven loop: launches iterations and checks the work flag every
// 'check' iterations (used when graph conditionals are unavailable)
cudaError_t wf_run_host_loop(const WfLaunch& L, WfCtl* host_ctl_pinned, const WfCtl* dev_ctl, cudaStream_t s,
                             double* kernel_ms) {
  constexpr int kCheck = 8;
  cudaEvent_t ev[kCheck][5] = {};
  cudaError_t e = cudaSuccess;
  if (kernel_ms)
    for (int k = 0; k < kCheck && e == cudaSuccess; k++)
      for (int q = 0; q < 5 && e == cudaSuccess; q++) e = cudaEventCreate(&ev[k][q]);
  for (int it = 0; it < (1 << 20) && e == cudaSuccess; it += kCheck) {
    for (int k = 0; k < kCheck; k++) {
      if (kernel_ms) cudaEventRecord(ev[k][0], s);
      launch_shade(L, s);
      if (kernel_ms) cudaEventRecord(ev[k][1], s);
      wf_extend<<<L.trace_blocks, 128, 0, s>>>();
      if (kernel_ms) cudaEventRecord(ev[k][2], s);
      wf_shadow<<<L.trace_blocks, 128, 0, s>>>();
      if (kernel_ms) cudaEventRecord(ev[k][3], s);
      wf_control<<<1, 1, 0, s>>>(0, 0);
      if (kernel_ms) cudaEventRecord(ev[k][4], s);
    }
    e = cudaMemcpyAsync(host_ctl_pinned, dev_ctl, sizeof(WfCtl), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) break;
    if (kernel_ms)
      for (int k = 0; k < kCheck; k++)
        for (int q = 0; q < 4; q++) {
          float ms = 0.0f;
          if (cudaEventElapsedTime(&ms, ev[k][q], ev[k][q + 1]) == cudaSuccess) kernel_ms[q] += ms;
        }
    if (!host_ctl_pinned->work) break;
  }
  if (kernel_ms)
    for (int k = 0; k < kCheck; k++)
      for (int q = 0; q < 5; q++)
        if (ev[k][q]) cudaEventDestroy(ev[k][q]);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t wf_resolve_launch(float* out, int n3, int accumulate, float sensor, cudaStream_t s) {
  wf_resolve<<<(n3 + 255) / 256, 256, 0, s>>>(out, n3, accumulate, sensor);
  return cudaGetLastError();
}

}  // namespace pr
