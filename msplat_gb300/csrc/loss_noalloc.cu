// SSIM + L1 training loss and its image gradient without any device
// allocation: msplat_loss_ssim_l1_noalloc.
//
// Who needs it: code that embeds the loss in a host which owns all device
// memory — an application with its own pool allocator, a serving or training
// process that has already reserved the GPU's memory, or a loop that must not
// take cudaMalloc's implicit device-wide synchronisation.  Such callers pass
// only their inputs and outputs; the loss's scratch (15 moment planes and 9
// derivative-field planes per pixel) and its three step scalars live in this
// file's static device arrays, which every GPU that loads the library holds
// until the process exits.
//
// Limit: at most kNoAllocMaxPixels = 512 * 512 = 262,144 pixels per image
// (24 floats per pixel: 25.2 MB of scratch).  Larger images are rejected.
//
// Sharing: every call on a device uses the same arrays, which keep the last
// call's contents.  Each call rewrites all the scratch it reads and zeroes the
// caller's loss output, so no state carries over between calls — but calls
// that overlap on the GPU (different streams, no ordering) race on the arrays.
//
// Set-up: the first call on each device looks up the arrays' device addresses
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "msplat_gb300.h"

namespace msplat {

constexpr long long kNoAllocMaxPixels = 512LL * 512LL;
constexpr int kNoAllocPlanes = 15 + 9;

static __device__ __align__(256) float g_noalloc_scratch[kNoAllocPlanes * kNoAllocMaxPixels];
static __device__ __align__(256) StepParams g_noalloc_params;

struct NoAllocDevice {
    bool ready = false;
    float *scratch = nullptr;
    StepParams *params = nullptr;
};

static NoAllocDevice g_noalloc_dev[64];
static std::mutex g_noalloc_mu;

// Device addresses of this device's copies of the arrays (looked up once per
// device; host code must not use the symbols' host-side names as addresses).
static int noalloc_setup(int dev, NoAllocDevice &out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.ready) {
        void *s = nullptr, *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&s, g_noalloc_scratch);
        if (e != cudaSuccess) {
            fprintf(stderr, "msplat_loss_ssim_l1_noalloc: cudaGetSymbolAddress(scratch): %s\n", cudaGetErrorString(e));
            return -4;
        }
        e = cudaGetSymbolAddress(&p, g_noalloc_params);
        if (e != cudaSuccess) {
            fprintf(stderr, "msplat_loss_ssim_l1_noalloc: cudaGetSymbolAddress(params): %s\n", cudaGetErrorString(e));
            return -4;
        }
        d.scratch = static_cast<float *>(s);
        d.params = static_cast<StepParams *>(p);
        d.ready = true;
    }
    out = d;
    return 0;
}

}  // namespace msplat

extern "C" int msplat_loss_ssim_l1_noalloc(const float *img, const uint8_t *gt, const uint8_t *mask, int width,
                                           int height, float ssim_weight, float loss_inv_n, float *v_img,
                                           float *loss_sum, void *stream) {
    using namespace msplat;
    if (!img || !gt || !v_img || !loss_sum) return -1;
    if (width <= 0 || height <= 0) return -2;
    const long long P = (long long)width * height;
    if (P > kNoAllocMaxPixels) {
        fprintf(stderr,
                "msplat_loss_ssim_l1_noalloc: %d x %d = %lld pixels exceeds the no-allocation limit of %lld pixels\n",
                width, height, P, kNoAllocMaxPixels);
        return -3;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) return -4;
    NoAllocDevice d;
    if (int rc = noalloc_setup(dev, d)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    StepParams sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.ssim_weight = ssim_weight;
    sp.loss_inv_n = loss_inv_n;
    sp.has_mask = mask ? 1 : 0;
    // pageable source: consumed by the time the call returns
    e = cudaMemcpyAsync(d.params, &sp, sizeof(sp), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(loss_sum, 0, sizeof(float), s);
    if (e != cudaSuccess) {
        fprintf(stderr, "msplat_loss_ssim_l1_noalloc: %s\n", cudaGetErrorString(e));
        return -5;
    }
    LossArgs la{};
    la.vt = single_view_table(0, width, height);
    la.num_tiles = la.vt.tile_base[1];
    la.sp = d.params;
    la.img = img;
    la.gt = gt;
    la.mask = mask;
    la.hbuf = d.scratch;             // 15 planes of P floats
    la.dbuf = d.scratch + 15 * P;    // 9 planes of P floats
    la.v_img = v_img;
    la.loss_sum = loss_sum;
    la.nan_counts = nullptr;
    launch_loss(la, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "msplat_loss_ssim_l1_noalloc: launch: %s\n", cudaGetErrorString(e));
        return -5;
    }
    return 0;
}
