// ajg_render_static: rendering for callers that cannot allocate device
// memory -- a host application whose device memory is owned by another
// allocator or fixed budget, or code that must not call cudaMalloc while it
// runs.  It renders exactly as ajg_render_device does, but its scratch (the
// film accumulators and one wave of path state) lives in the file-scope
// device array below instead of the context's wave arena and a per-call
// film allocation.
//
// The array is reserved on every GPU that loads this library, for as long
// as the process runs.  All calls on a device share it and it keeps the
// previous call's contents, so each call clears the film part before use,
// and calls whose GPU work overlaps (different streams, or several contexts
// on one device) race on it.  Every launch of a call is ordered on the
// caller's stream: the traversal launches the context overlaps on its trace
// stream are forked from that stream and joined back into it by events.
#include <mutex>
#include <string>

#include "scene.cuh"

namespace {

// 32 MiB: 32 bytes per film pixel plus a wave of at least 1,024 paths.
constexpr uint64_t kStaticScratchBytes = 32ull << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

}  // namespace

extern "C" {

// The host cannot pass g_static_scratch itself (in host code the name is a
// stand-in, not a device address): the device address is looked up once per
// device, with that device current, on the first call there.  That first
// call therefore loads the module on the device and should come before any
// stream capture.
int ajg_render_static(ajg_scene* scene, const ajg_camera* cam,
                      const ajg_render_params* params, float* d_out_rgbw,
                      void* stream) {
  if (!scene || !cam || !params || !d_out_rgbw) return AJG_ERR_INVALID;
  ajg_ctx* ctx = scene->ctx;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (ctx->device < 0 || ctx->device >= kMaxDevices) {
    ctx->last_error = "render_static: device ordinal above 63";
    return AJG_ERR_UNSUPPORTED;
  }
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) {
    ctx->last_error = std::string("render_static: ") + cudaGetErrorString(e);
    return AJG_ERR_CUDA;
  }
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> g(g_scratch_mu);
    if (!g_scratch_addr[ctx->device]) {
      e = cudaGetSymbolAddress(&g_scratch_addr[ctx->device], g_static_scratch);
      if (e != cudaSuccess) {
        g_scratch_addr[ctx->device] = nullptr;
        ctx->last_error =
            std::string("render_static: scratch address: ") +
            cudaGetErrorString(e);
        return AJG_ERR_CUDA;
      }
    }
    base = g_scratch_addr[ctx->device];
  }
  int rc = ajg::render_in_scratch(scene, *cam, *params,
                                  reinterpret_cast<float4*>(d_out_rgbw),
                                  static_cast<cudaStream_t>(stream),
                                  static_cast<char*>(base), kStaticScratchBytes);
  if (rc) return rc;
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    ctx->last_error = std::string("render_static: ") + cudaGetErrorString(e);
    return AJG_ERR_CUDA;
  }
  return AJG_OK;
}

}  // extern "C"
