// pr_render_dev_noalloc: the plain (megakernel) render for callers that must
// not allocate device memory while they render.
//
// Who needs it: frame loops with a hard time budget (cudaMalloc / cudaFree
// can synchronise the whole device and stall the frame), and host
// applications whose device memory is all handed out by their own pool
// allocator, where an allocation behind the pool's back can fail or break
// its accounting.  pr_render_dev grows its scratch on demand with
// cudaMalloc; this entry point never does.
//
// Its scratch -- the per-chunk partial images of the megakernel and the
// device error word / counters -- lives in one file-scope __device__ array
// of kNoAllocScratchBytes (16 MiB), which every GPU that loads this library
// keeps for the life of the process.  The first call on a device looks up
// the array's device address with cudaGetSymbolAddress (with that device
// current); make that first call before any stream capture begins.  The
// scene still comes from pr_scene_upload, which does allocate, at set-up.
//
// The address is looked up once per device number and kept: it is the
// array's address in that device's primary context, the one the CUDA
// runtime uses.  It is not valid in a context the caller made itself with
// the driver API, nor after cudaDeviceReset (the array then has a new
// address that this library does not look up again).
//
// All calls share the one array: two calls whose work overlaps on the GPU
// (different streams or contexts on the same device) race on it and give
// wrong images.  Each call clears the error word and counters it uses; the
// partial images are fully overwritten by every call.
//
// Sample chunks: pr_render_dev splits each pixel's samples into
// min(ceil(1.2e6 / pixels), spp) chunks, each summed by its own thread.
// This entry point keeps that split while the chunks' partial images fit in
// the array and otherwise uses as many chunks as fit (for example one
// instead of two at 1024 x 768).  The samples are the same, only the order
// of the float sums differs, so such images agree with pr_render_dev's to
// float rounding, not bit for bit.
#include <cuda_runtime.h>

#include <mutex>

#include "ctx_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB
constexpr size_t kNoAllocHeader = 256;                 // error word + counters
constexpr int kMaxDevices = 64;

// host code only sees a stand-in for this symbol; its device address comes
// from cudaGetSymbolAddress
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// once per device, with that device current
cudaError_t scratch_for_device(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[device]);
  return cudaSuccess;
}

}  // namespace

extern "C" int pr_render_dev_noalloc(pr_ctx* c, const pr_camera* cam, const pr_render_params* p, float* rgb_dev,
                                     uint64_t sample_offset, int accumulate) {
  using namespace pr;
  if (!c) return PR_E_ARG;
  if (!cam || !p) return ctx_fail(c, PR_E_ARG, "null camera or parameters");
  if (!c->scene_ready) return ctx_fail(c, PR_E_SCENE, "no scene uploaded");
  if (!rgb_dev) return ctx_fail(c, PR_E_ARG, "null output");
  if (p->mode != PR_MODE_MEGAKERNEL)
    return ctx_fail(c, PR_E_UNSUPPORTED, "pr_render_dev_noalloc renders the megakernel form only");
  if (c->cur.kerr.enabled) return ctx_fail(c, PR_E_UNSUPPORTED, "pr_render_dev_noalloc renders straight-ray scenes only");
  RenderCfg g;
  int st = prepare_render(c, cam, p, sample_offset, g);
  if (st != PR_OK) return st;
  const size_t n3 = (size_t)g.width * g.height * 3;
  const size_t room = kNoAllocScratchBytes - kNoAllocHeader;
  const size_t max_pixels = room / (3 * sizeof(float));
  if ((size_t)g.width * g.height > max_pixels)
    return ctx_fail(c, PR_E_ARG,
                    "image of " + std::to_string(g.width) + "x" + std::to_string(g.height) +
                        " pixels exceeds the allocation-free scratch (at most " + std::to_string(max_pixels) +
                        " pixels); use pr_render_dev");
  // fewer sample chunks if their partial images would not fit
  g.chunks = std::max(1, std::min(g.chunks, (int)(room / (n3 * sizeof(float)))));
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return ctx_fail(c, PR_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  cudaGetLastError();  // an error left by an unrelated earlier call is not this call's
  unsigned char* base = nullptr;
  e = scratch_for_device(c->device, &base);
  if (e != cudaSuccess)
    return ctx_fail(c, PR_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  uint32_t* err = reinterpret_cast<uint32_t*>(base);
  unsigned long long* counters = reinterpret_cast<unsigned long long*>(base + 64);
  float* partial = reinterpret_cast<float*>(base + kNoAllocHeader);
#define NA_CUDA(call)                                                                           \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return ctx_fail(c, PR_E_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)
  NA_CUDA(cudaMemsetAsync(base, 0, kNoAllocHeader, c->stream));
  NA_CUDA(cudaEventRecord(c->ev0, c->stream));
  NA_CUDA(launch_megakernel(c->cur.dev, g, partial, err, counters, c->stream));
  NA_CUDA(launch_reduce(partial, rgb_dev, (int)n3, g.chunks, accumulate, c->stream));
  NA_CUDA(cudaEventRecord(c->ev1, c->stream));
  uint32_t bits = 0;
  unsigned long long cnt[4] = {0, 0, 0, 0};
  NA_CUDA(cudaMemcpyAsync(&bits, err, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
  NA_CUDA(cudaMemcpyAsync(cnt, counters, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  NA_CUDA(cudaStreamSynchronize(c->stream));
#undef NA_CUDA
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->stats = pr_render_stats{cnt[0], cnt[1], cnt[2], cnt[3], ms, 2};
  if (bits) return ctx_fail(c, PR_E_DEVICE, device_error_message(bits));
  return PR_OK;
}
