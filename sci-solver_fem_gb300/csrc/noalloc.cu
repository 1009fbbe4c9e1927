// noalloc.cu -- femgpu_load_vector_device_noalloc: the load vector on device arrays
// with its per-element scratch in a region compiled into the library, so the call
// makes no device allocation.
//
// The region sits in its own translation unit: with CUDA's lazy module loading it is
// reserved only when a process first uses this entry point.
#include <mutex>

#include "context.cuh"

using namespace femgpu;

struct femgpu_ctx : Ctx {};

namespace {

constexpr int64_t kMaxElements = FEMGPU_NOALLOC_MAX_ELEMENTS;
constexpr int kMaxDevices = 64;

// [0, kMaxElements): per-element measure / (k (k + 1)); [kMaxElements, 2 kMaxElements):
// per-element sum of f over the element's vertices.
static __device__ __align__(256) double g_load_scratch[2 * kMaxElements];

std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of the region on the current device `dev`, looked up once per device.
double* scratch_on(int dev) {
  FG_REQUIRE(dev >= 0 && dev < kMaxDevices, FEMGPU_ERR_LIMIT, "device ordinal beyond the no-alloc table");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_load_scratch);
    FG_REQUIRE(e == cudaSuccess && p != nullptr, FEMGPU_ERR_CUDA,
               std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  return g_scratch_ptr[dev];
}

}  // namespace

extern "C" femgpu_status femgpu_load_vector_device_noalloc(femgpu_handle h, const double* d_f, double* d_b) {
  if (!h || !d_f || !d_b) return FEMGPU_ERR_INVALID;
  try {
    FG_CUDA(cudaSetDevice(h->device));
    FG_REQUIRE(h->has_mesh, FEMGPU_ERR_NOT_READY, "femgpu_set_mesh first");
    FG_REQUIRE(h->mesh.ne <= kMaxElements, FEMGPU_ERR_LIMIT,
               "mesh has more elements than the no-alloc scratch holds (FEMGPU_NOALLOC_MAX_ELEMENTS)");
    double* base = scratch_on(h->device);
    load_vector_enqueue(*h, d_f, d_b, base, base + kMaxElements);
    return FEMGPU_OK;
  } catch (const Error& e) {
    h->last_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    h->last_error = e.what();
    return FEMGPU_ERR_INVALID;
  }
}
