// SSIM + L1 training loss and its image gradient without any device
// allocation: msplat_loss_ssim_l1_noalloc.
//
// Who needs it: code that embeds the loss in a host which owns all device
// memory — an application with its own pool allocator, a serving or training
// process that has already reserved the GPU's memory, or a loop that must not
// take cudaMalloc's implicit device-wide synchronisation.  Such callers pass
// only their inputs and outputs.  The loss kernel keeps all its intermediates
// in shared memory, so the only device state is the three step scalars, in
// this file's static device copy of StepParams, which every GPU that loads
// the library holds until the process exits.  Any image size.
//
// Sharing: every call on a device uses the same scalars, rewritten in stream
// order by a one-thread kernel (the values travel as kernel arguments, so no
// host buffer is read after the call returns) before the loss kernel runs,
// and each call zeroes the caller's loss output, so no state carries over
// between calls — but calls that overlap on the GPU (different streams, no
// ordering) race on the scalars.
//
// Set-up: the first call on each device looks up the scalars' device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture.
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "msplat_gb300.h"

namespace msplat {

static __device__ __align__(256) StepParams g_noalloc_params;

struct NoAllocDevice {
    bool ready = false;
    StepParams *params = nullptr;
};

static NoAllocDevice g_noalloc_dev[64];
static std::mutex g_noalloc_mu;

// Device address of this device's copy of the scalars (looked up once per
// device; host code must not use the symbol's host-side name as an address).
static int noalloc_setup(int dev, NoAllocDevice &out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.ready) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_params);
        if (e != cudaSuccess) {
            fprintf(stderr, "msplat_loss_ssim_l1_noalloc: cudaGetSymbolAddress(params): %s\n", cudaGetErrorString(e));
            return -4;
        }
        d.params = static_cast<StepParams *>(p);
        d.ready = true;
    }
    out = d;
    return 0;
}

// Writes the call's scalars into the shared device copy (one thread).
__global__ void k_noalloc_scalars(StepParams *p, float ssim_weight, float loss_inv_n, int has_mask,
                                  float *loss_sum) {
    p->ssim_weight = ssim_weight;
    p->loss_inv_n = loss_inv_n;
    p->has_mask = has_mask;
    *loss_sum = 0.f;
}

}  // namespace msplat

extern "C" int msplat_loss_ssim_l1_noalloc(const float *img, const uint8_t *gt, const uint8_t *mask, int width,
                                           int height, float ssim_weight, float loss_inv_n, float *v_img,
                                           float *loss_sum, void *stream) {
    using namespace msplat;
    if (!img || !gt || !v_img || !loss_sum) return -1;
    if (width <= 0 || height <= 0) return -2;
    if ((long long)width * height > 0x7fffffffLL || (height + 31) / 32 > 65535) {
        fprintf(stderr, "msplat_loss_ssim_l1_noalloc: %d x %d is beyond the kernel's grid\n", width, height);
        return -3;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) return -4;
    NoAllocDevice d;
    if (int rc = noalloc_setup(dev, d)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    k_noalloc_scalars<<<1, 1, 0, s>>>(d.params, ssim_weight, loss_inv_n, mask ? 1 : 0, loss_sum);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "msplat_loss_ssim_l1_noalloc: %s\n", cudaGetErrorString(e));
        return -5;
    }
    LossArgs la{};
    la.vt = single_view_table(0, width, height);
    la.sp = d.params;
    la.img = img;
    la.gt = gt;
    la.mask = mask;
    la.v_img = v_img;
    la.loss_sum = loss_sum;
    la.nan_counts = nullptr;
    if (launch_loss(la, s) < 0) return -4;
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "msplat_loss_ssim_l1_noalloc: launch: %s\n", cudaGetErrorString(e));
        return -5;
    }
    return 0;
}
