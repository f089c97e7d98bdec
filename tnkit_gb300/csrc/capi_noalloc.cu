// tnk_apply_two_site_f64_noalloc: the two-site H_eff matvec for callers that cannot allocate
// device memory.
//
// Some callers cannot call cudaMalloc at the point where they need a matvec: code running inside
// a host callback or a signal-safe section, a driver of a pre-sized memory pool that must not
// grow, an embedding that forbids allocation after start-up, or a foreign-language binding that
// has no device allocator of its own. They still own the inputs and the output, but cannot
// provide the stage-1/stage-2 workspace that tnk_apply_two_site_f64 takes. This entry point uses
// a fixed scratch array that lives in the library's own device memory instead.
//
// The scratch is a file-scope __device__ array of TNK_NOALLOC_SCRATCH_ELEMS doubles (64 MiB).
// Every GPU on which the library's module is loaded holds it until the process exits. Host code
// must not use the array's name as a device pointer (on the host it names a stand-in object), so
// the first call on each device looks its device address up with cudaGetSymbolAddress, with that
// device current, and caches it; that first call should therefore come before any stream capture.
// The cached address belongs to the device's current primary context: after cudaDeviceReset (or
// anything else that destroys that context) the module is loaded again at a new address and the
// cached one is stale, so a process that resets a device must not call this entry point on it
// again.
// Every call shares the one array, which keeps the previous call's contents: calls that overlap
// on the GPU (different streams, or threads, without ordering between them) race on it. Nothing
// in the scratch needs to start at zero: every element a call reads is first written by that
// call (stage 1 writes each intermediate block stage 2 reads, stage 2 writes every slice of each
// block stage 3 reads, stage 3 writes every split-K partial stage 4 sums). The entry point
// allocates nothing: no cudaMalloc, no cudaFree, no allocating library routine.
#include <mutex>

#include "tnk_internal.cuh"

#define TNK_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[TNK_NOALLOC_SCRATCH_ELEMS];

namespace {

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[TNK_NOALLOC_MAX_DEVICES] = {};

// The device address of the scratch array on the current device (looked up once per device).
int scratch_on_current_device(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        tnk::set_error("noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
        return TNK_ERR_DEVICE;
    }
    if (dev < 0 || dev >= TNK_NOALLOC_MAX_DEVICES) {
        tnk::set_error("noalloc: device %d out of range", dev);
        return TNK_ERR_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            tnk::set_error("noalloc: cudaGetSymbolAddress on device %d: %s", dev,
                           cudaGetErrorString(e));
            return TNK_ERR_DEVICE;
        }
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return TNK_OK;
}

}  // namespace

extern "C" int tnk_noalloc_scratch_elems(int64_t* out) {
    if (!out) return TNK_ERR_ARG;
    *out = (int64_t)TNK_NOALLOC_SCRATCH_ELEMS;
    return TNK_OK;
}

extern "C" int tnk_apply_two_site_f64_noalloc(const tnk_plan3* plan, const double* L,
                                              const double* theta, const double* R,
                                              double* out, void* stream) {
    if (!plan || !L || !theta || !R || !out) {
        tnk::set_error("apply_two_site_noalloc: null plan, operand or output");
        return TNK_ERR_ARG;
    }
    if (plan->ws1_elems < 0 || plan->ws2_elems < 0) {
        tnk::set_error("apply_two_site_noalloc: negative workspace sizes in the plan");
        return TNK_ERR_ARG;
    }
    const int64_t need = plan->ws1_elems + plan->ws2_elems;
    if (need > (int64_t)TNK_NOALLOC_SCRATCH_ELEMS) {
        tnk::set_error("apply_two_site_noalloc: the plan needs %lld scratch doubles, the fixed "
                       "scratch holds %lld (TNK_NOALLOC_SCRATCH_ELEMS); use "
                       "tnk_apply_two_site_f64 with a caller workspace",
                       (long long)need, (long long)TNK_NOALLOC_SCRATCH_ELEMS);
        return TNK_ERR_SIZE;
    }
    double* ws = nullptr;
    int rc = scratch_on_current_device(&ws);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    tnk::Slots s{{L, theta, R, ws}};
    rc = tnk::launch_gemm_f64(plan->t1, plan->s1, plan->tiles1, plan->n_tiles1, s, ws, st);
    if (rc) return rc;
    rc = tnk::launch_comb_f64(plan->t2, plan->c2, plan->items2, plan->n_items2, ws, ws, st);
    if (rc) return rc;
    rc = tnk::launch_gemm_f64(plan->t3, plan->s3, plan->tiles3, plan->n_tiles3, s, out, st);
    if (rc) return rc;
    return tnk::launch_comb_f64(plan->t4, plan->c4, plan->items4, plan->n_items4, ws, out, st);
}
