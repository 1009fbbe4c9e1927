// noalloc.cu -- femgpu_load_vector_device_noalloc: the load vector on device arrays
// with its per-element scratch in a region compiled into the library, so the call
// makes no device allocation.
//
// The region sits in its own translation unit: under CUDA's lazy module loading (the
// default since CUDA 12.2) it is reserved only when a process first uses this entry
// point; with CUDA_MODULE_LOADING=EAGER every context that loads the library reserves it.
#include "context.cuh"

using namespace femgpu;

struct femgpu_ctx : Ctx {};

namespace {

constexpr int64_t kMaxElements = FEMGPU_NOALLOC_MAX_ELEMENTS;

// [0, kMaxElements): per-element measure / (k (k + 1)); [kMaxElements, 2 kMaxElements):
// per-element sum of f over the element's vertices.
static __device__ __align__(256) double g_load_scratch[2 * kMaxElements];

// Device address of the region in the handle's context, looked up on the handle's first
// call (its device is current).  The address belongs to the context that loaded this
// module, and a handle never outlives its context, so it stays valid for the handle.
double* scratch_of(femgpu_ctx* h) {
  if (!h->noalloc_scratch) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_load_scratch);
    FG_REQUIRE(e == cudaSuccess && p != nullptr, FEMGPU_ERR_CUDA,
               std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
    h->noalloc_scratch = static_cast<double*>(p);
  }
  return h->noalloc_scratch;
}

}  // namespace

extern "C" femgpu_status femgpu_load_vector_device_noalloc(femgpu_handle h, const double* d_f, double* d_b) {
  if (!h || !d_f || !d_b) return FEMGPU_ERR_INVALID;
  try {
    FG_CUDA(cudaSetDevice(h->device));
    FG_REQUIRE(h->has_mesh, FEMGPU_ERR_NOT_READY, "femgpu_set_mesh first");
    FG_REQUIRE(h->mesh.ne <= kMaxElements, FEMGPU_ERR_LIMIT,
               "mesh has more elements than the no-alloc scratch holds (FEMGPU_NOALLOC_MAX_ELEMENTS)");
    double* base = scratch_of(h);
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
