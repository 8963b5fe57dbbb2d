// Host driver of the GB300 training step: a grow-only device arena sized by
// the largest view and Gaussian count seen, one CUDA stream, and the stage
// order of msplat_train_step (core/metal/msplat_metal.mm:1118-1740).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "kernels.h"
#include "msplat_engine.h"

namespace msplat {

#define CK(x)                                                                                  \
    do {                                                                                       \
        cudaError_t err_ = (x);                                                                \
        if (err_ != cudaSuccess)                                                               \
            throw std::runtime_error(std::string(#x) + ": " + cudaGetErrorString(err_));       \
    } while (0)

static const bool g_sync_check = getenv("MSPLAT_SYNC_CHECK") != nullptr;

void debug_sync(cudaStream_t s, const char *what) {
    if (!g_sync_check) return;
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string("kernel ") + what + ": " + cudaGetErrorString(e));
}

struct Buf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

// The step scalars of every view as one kernel argument: the upload before
// each step (or graph replay) is a kernel launch on the engine's stream, not
// a copy-engine transfer between the previous step's kernels and the next.
struct ParamsPack {
    StepParams p[kMaxViews];
};
static_assert(sizeof(ParamsPack) <= 32000, "kernel argument size");
static_assert(sizeof(StepParams) % 4 == 0, "StepParams is copied in words");

__global__ void __launch_bounds__(256) k_set_params(StepParams *dst, const __grid_constant__ ParamsPack pk, int words) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(&pk);
    uint32_t *d = reinterpret_cast<uint32_t *>(dst);
    for (int i = threadIdx.x; i < words; i += blockDim.x) d[i] = src[i];
}

// n floats to page-locked host memory (through its device mapping)
__global__ void k_copy_out(float *dst, const float *src, int n) {
    if ((int)threadIdx.x < n) dst[threadIdx.x] = src[threadIdx.x];
}

class Engine {
  public:
    explicit Engine(int device) : device_(device) {
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) {
            CK(cudaEventCreateWithFlags(&stage_ready_[k], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&stage_free_[k], cudaEventDisableTiming));
            CK(cudaEventRecord(stage_free_[k], stream_));
        }
        cudaDeviceProp prop;
        CK(cudaGetDeviceProperties(&prop, device));
        num_sms_ = prop.multiProcessorCount;
        for (auto &row : ev_)
            for (auto &ev : row) CK(cudaEventCreate(&ev));
        for (auto &ev : marker_) CK(cudaEventCreate(&ev));
    }
    ~Engine() {
        cudaSetDevice(device_);
        cudaStreamSynchronize(stream_);
        clear_graphs();
        for (auto &kv : bufs_) cudaFree(kv.second.ptr);
        for (auto &row : ev_)
            for (auto &ev : row) cudaEventDestroy(ev);
        for (auto &ev : marker_) cudaEventDestroy(ev);
        cudaStreamSynchronize(copy_stream_);
        for (int k = 0; k < 2; k++) {
            cudaEventDestroy(stage_ready_[k]);
            cudaEventDestroy(stage_free_[k]);
        }
        cudaStreamDestroy(copy_stream_);
        cudaStreamDestroy(stream_);
    }

    void reserve_points(int n) { ensure_points(n); }

    void train_step(const MsplatGaussians &g, const MsplatAdamState *st, const MsplatStepArgs &args, const uint8_t *gt,
                    const uint8_t *mask, bool backward) {
        const uint8_t *gts[1] = {gt}, *masks[1] = {mask};
        run_views(g, st, &args, 1, gt ? gts : nullptr, masks, backward);
    }

    // Copies host images into engine-owned device buffers on the engine's
    // stream (asynchronous for page-locked sources), then runs the step.
    // The copies run on a second stream into two alternating stage buffers,
    // so a step's upload overlaps the step before it: the engine stream waits
    // for this step's copy, and a buffer is refilled only after the step that
    // read it.  Asynchronous for page-locked sources.
    void train_step_host(const MsplatGaussians &g, const MsplatAdamState *st, const MsplatStepArgs &args,
                         const uint8_t *gt_host, const uint8_t *mask_host) {
        CK(cudaSetDevice(device_));
        const size_t P = (size_t)args.width * args.height;
        const int k = stage_slot_;
        stage_slot_ ^= 1;
        const std::string gname = k ? "gt_stage1" : "gt_stage0", mname = k ? "mask_stage1" : "mask_stage0";
        alloc(gname.c_str(), P * 3);
        if (mask_host) alloc(mname.c_str(), P);
        CK(cudaStreamWaitEvent(copy_stream_, stage_free_[k], 0));   // the step that last read this buffer is done
        CK(cudaMemcpyAsync(ptr<uint8_t>(gname.c_str()), gt_host, P * 3, cudaMemcpyHostToDevice, copy_stream_));
        const uint8_t *mask_d = nullptr;
        if (mask_host) {
            CK(cudaMemcpyAsync(ptr<uint8_t>(mname.c_str()), mask_host, P, cudaMemcpyHostToDevice, copy_stream_));
            mask_d = ptr<uint8_t>(mname.c_str());
        }
        CK(cudaEventRecord(stage_ready_[k], copy_stream_));
        CK(cudaStreamWaitEvent(stream_, stage_ready_[k], 0));
        train_step(g, st, args, ptr<uint8_t>(gname.c_str()), mask_d, true);
        CK(cudaEventRecord(stage_free_[k], stream_));
    }

    // Copies the last step's per-view loss sums (loss_sum[v], v < views; the
    // loss is the sum over the view's pixel count) to `dst` on the engine's
    // stream without waiting: page-locked `dst` is filled when the stream
    // gets there.
    void loss_async(float *dst) {
        const int n = std::max(1, last_views_);
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, dst) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
            // page-locked: a one-warp kernel writes through the mapping (no
            // copy-engine transfer on the step stream)
            k_copy_out<<<1, 32, 0, stream_>>>(static_cast<float *>(at.devicePointer), ptr<float>("loss_sum"), n);
            CK(cudaGetLastError());
        } else {
            cudaGetLastError();   // an unregistered pointer is not an error here
            CK(cudaMemcpyAsync(dst, ptr<float>("loss_sum"), sizeof(float) * n, cudaMemcpyDefault, stream_));
        }
    }

    // Multi-view step: B views (any sizes) rendered and back-propagated by
    // the same launches as one view (each stage covers all views), each
    // view's image gradient scaled by 1/B so the parameter gradients are the
    // views' mean, then one optimizer update with the scalars of args[0]: the
    // 4-group Adam with the regularizer, the SH Adam (fused in the projection
    // backward) over Gaussians visible in any view, and SGLD.
    void train_step_batch(const MsplatGaussians &g, const MsplatAdamState &st, const MsplatStepArgs *args, int B,
                          const uint8_t *const *gts, const uint8_t *const *masks) {
        if (B <= 0) throw std::runtime_error("batch of no views");
        if (B > kMaxViews) throw std::runtime_error("more than 16 views in one step");
        for (int v = 0; v < B; v++)
            if (!gts || !gts[v]) throw std::runtime_error("multi-view step without a target image");
        run_views(g, &st, args, B, gts, masks, true);
    }

  private:
    // One step over B views; gts == nullptr renders only (one view).
    void run_views(const MsplatGaussians &g, const MsplatAdamState *st, const MsplatStepArgs *args, int B,
                   const uint8_t *const *gts, const uint8_t *const *masks, bool backward) {
        CK(cudaSetDevice(device_));
        int w[kMaxViews], h[kMaxViews];
        for (int v = 0; v < B; v++) {
            validate(g, args[v]);
            w[v] = args[v].width;
            h[v] = args[v].height;
        }
        const int N = g.num_points;
        if ((long long)N * B >= (1LL << 31)) throw std::runtime_error("views x Gaussians exceeds 2^31 records");
        const ViewTable vt = make_view_table(N, B, w, h);
        const int T = vt.tile_base[B];
        const long long P = vt.pix_base[B];
        if (P > (1LL << 31) / 16) throw std::runtime_error("views too large for one step");
        const long long legacy = std::max<long long>(48LL * N * B, 1);   // msplat_metal.mm:1142 legacy capacity, per view
        const MsplatTuning tune = tuning_;
        // each view's depth chunks from its own tiles, mode and the one-view
        // capacity (as the reference, which steps one view at a time); the
        // raster launches cover runs of consecutive views with the same K
        int Kv[kMaxViews];
        int K = 1;
        for (int v = 0; v < B; v++) {
            Kv[v] = choose_k(args[v], vt.tile_base[v + 1] - vt.tile_base[v], std::max<long long>(48LL * N, 1), tune);
            K = std::max(K, Kv[v]);
        }
        const std::vector<RasterRun> runs = raster_runs(vt, Kv);
        long long chunk_entries = 0;
        for (const RasterRun &r : runs) chunk_entries += r.k > 1 ? r.k * (vt.pix_base[r.v1] - vt.pix_base[r.v0]) : 0;
        // fixed intersection budget (monolithic raster only, as in the
        // reference): a view that does not fit is rastered in tile groups
        const bool fixed = isect_slots_ > 0 && K == 1;
        const long long cap = fixed ? isect_slots_ : legacy;
        // slots are addressed with 32-bit offsets and indices
        if (cap >= (1LL << 31)) throw std::runtime_error("intersection buffer of 2^31 slots or more");
        const bool has_gt = gts != nullptr;
        ensure_points(N, B);
        ensure_tiles(T);
        ensure_isect(cap);
        ensure_pixels(P);
        if (chunk_entries > 0) ensure_chunks(chunk_entries);
        last_T_ = T;
        last_K_ = K;
        last_views_ = B;
        for (int v = 0; v < B; v++) last_view_P_[v] = (long long)w[v] * h[v];
        if (timing_) slot_ = (timed_steps_++) % kRing;

        ParamsPack pack;
        std::memset(&pack, 0, sizeof(pack));
        StepParams *sps = pack.p;
        for (int v = 0; v < B; v++) {
            const uint8_t *mk = (has_gt && masks) ? masks[v] : nullptr;
            fill_params(args[v], sps[v], mk != nullptr);
            sps[v].gt = has_gt ? gts[v] : nullptr;
            sps[v].mask = mk;
            if (B > 1) sps[v].loss_inv_n = args[v].loss_inv_n / (float)B;
        }
        // The upload stays outside any captured graph: kernels read the
        // scalars through this device block, so a replay sees this step's
        // values.  A plain launch: it runs after the previous step's kernels
        // (which read the block) have finished.
        k_set_params<<<1, 256, 0, stream_>>>(ptr<StepParams>("params"), pack,
                                             (int)(sizeof(StepParams) * B / 4));
        CK(cudaGetLastError());
        launches_ += 1;
        // every buffer the step touches exists now (sized above), so a capture
        // below allocates nothing
        const size_t cb = tile_cta_bins_bytes(vt);
        if (cb) alloc("cta_bins", cb);
        const bool presorted = tune.tile_order == 1 && cb > 0 && N > 0;
        if (presorted) {
            const size_t recs = (size_t)N * B;
            alloc("gs_key0", 4 * recs); alloc("gs_key1", 4 * recs);
            alloc("gs_val0", 4 * recs); alloc("gs_val1", 4 * recs);
            alloc("gs_hist", 4 * (size_t)B * kGsDigits * ((N + kGsPerCta - 1) / kGsPerCta));
            alloc("gs_dtot", 4 * (size_t)B * kGsDigits);
            alloc("srect", 8 * recs);
            alloc("rect", 8 * recs);
        }
        const MsplatStepArgs &a0 = args[0];
        const bool opt = a0.do_optimizer && st;

        auto issue = [&]() {
        // kernels of this step, one launch per stage whatever the views:
        // projection, the tile-mapping and loss launches (counted where they
        // are issued), raster (+ merge when chunked), and for training raster
        // backward (+ prefix/suffix), projection backward, Adam, SGLD
        long long raster_launches = 0;
        for (const RasterRun &r : runs) raster_launches += r.k > 1 ? 2 : 1;
        launches_ += 1 + raster_launches;
        // (the one-view projection backward is two launches with the optimizer:
        // the VJP, then the SH Adam walk)
        if (has_gt && backward)
            launches_ += raster_launches + 1 + (opt && B == 1 ? 1 : 0) + (opt ? 1 : 0) + (a0.do_sgld ? 1 : 0);
        CK(cudaMemsetAsync(ptr<uint32_t>("tile_counts"), 0, sizeof(uint32_t) * 2 * (size_t)T, stream_));
        CK(cudaMemsetAsync(ptr<float>("loss_sum"), 0, sizeof(float) * B, stream_));

        mark(0);
        ProjectArgs pa{};
        pa.vt = vt; pa.rest_bases = g.rest_bases;
        pa.means = g.means; pa.scales = g.scales; pa.quats = g.quats;
        pa.features_dc = g.features_dc; pa.features_rest = g.features_rest; pa.opacities = g.opacities;
        pa.sp = ptr<StepParams>("params");
        pa.rec = ptr<SplatRec>("rec"); pa.depths = ptr<float>("depths"); pa.radii = ptr<int>("radii");
        pa.aabb = ptr<float2>("aabb"); pa.tiles_hit = ptr<int>("tiles_hit");
        pa.rect = presorted ? ptr<ushort4>("rect") : nullptr;
        pa.grad = backward ? ptr<GradRec>("grad") : nullptr;
        pa.nan_counts = ptr<unsigned>("nan_counts");
        launch_project_fwd(pa, stream_);
        debug_sync(stream_, "project_fwd");
        mark(1);

        TileArgs ta{};
        ta.vt = vt; ta.num_tiles = T; ta.capacity = cap; ta.sort_width = tune.sort_width;
        ta.radii = pa.radii; ta.depths = pa.depths; ta.rec = pa.rec; ta.aabb = pa.aabb; ta.rect = pa.rect;
        ta.tile_counts = ptr<uint32_t>("tile_counts"); ta.tile_write = ta.tile_counts + T;
        ta.tile_offsets = ptr<uint32_t>("tile_offsets"); ta.max_tile_count = ptr<uint32_t>("max_tile");
        ta.keys = ptr<uint64_t>("keys"); ta.keys_alt = ptr<uint64_t>("keys_alt");
        ta.isect_ids = ptr<uint32_t>("isect_ids"); ta.nan_counts = pa.nan_counts;
        ta.cta_bins = cb ? ptr<uint32_t>("cta_bins") : nullptr;
        ta.tile_lists = ptr<uint32_t>("tile_lists"); ta.tile_class = ptr<uint32_t>("tile_class");
        ta.tile_lo = 0; ta.tile_hi = T; ta.isect_lo = 0;
        ta.sort_width = tune.sort_width;
        ta.presorted = presorted ? 1 : 0;
        if (presorted) {
            ta.gs_key[0] = ptr<uint32_t>("gs_key0"); ta.gs_key[1] = ptr<uint32_t>("gs_key1");
            ta.gs_val[0] = ptr<uint32_t>("gs_val0"); ta.gs_val[1] = ptr<uint32_t>("gs_val1");
            ta.gs_hist = ptr<uint32_t>("gs_hist"); ta.srect = ptr<ushort4>("srect");
            ta.gs_dtot = ptr<uint32_t>("gs_dtot");
        }
        std::vector<TileGroup> groups;
        if (!fixed) {
            launches_ += launch_tiles(ta, num_sms_, stream_);
        } else {
            // the group boundaries need the tile counts on the host
            launches_ += launch_tile_count(ta, stream_);
            std::vector<uint32_t> counts((size_t)T);
            CK(cudaMemcpyAsync(counts.data(), ta.tile_counts, sizeof(uint32_t) * (size_t)T, cudaMemcpyDeviceToHost,
                               stream_));
            CK(cudaStreamSynchronize(stream_));
            groups = tile_groups(counts, cap);
        }
        last_groups_ = fixed ? (int)groups.size() : 1;
        // (re)build the lists of one tile group; every build after the first
        // re-zeroes the scatter's write counters and the sorts' work counters
        int builds = 0;
        auto build_group = [&](const TileGroup &gr) {
            TileArgs tg = ta;
            tg.tile_lo = gr.lo; tg.tile_hi = gr.hi; tg.isect_lo = gr.base;
            if (builds++ > 0) {
                CK(cudaMemsetAsync(ta.tile_write, 0, sizeof(uint32_t) * (size_t)T, stream_));
                CK(cudaMemsetAsync(ta.tile_class + 4, 0, sizeof(uint32_t) * 4, stream_));
            }
            launches_ += launch_tile_build(tg, num_sms_, stream_);
        };
        mark(2);

        RasterArgs ra{};
        ra.vt = vt; ra.num_tiles = T; ra.k_max = K; ra.capacity = cap; ra.tile_lo = 0; ra.isect_lo = 0;
        ra.chunk = tune.chunk; ra.batch = tune.raster_batch; ra.bwd_px = tune.bwd_pixels; ra.split = tune.tile_split;
        ra.sp = pa.sp; ra.tile_offsets = ta.tile_offsets; ra.isect_ids = ta.isect_ids;
        ra.n = (uint32_t)((long long)N * B); ra.rec = pa.rec;
        ra.out_img = ptr<float>("out_img"); ra.final_T = ptr<float>("final_T"); ra.final_idx = ptr<int>("final_idx");
        ra.chunk_p0 = 0; ra.chunk_P = P;
        ra.v_img = ptr<float>("v_img"); ra.grad = ptr<GradRec>("grad"); ra.nan_counts = pa.nan_counts;
        auto group_raster = [&](const TileGroup &gr) {
            RasterArgs rg = ra;
            rg.tile_lo = gr.lo; rg.num_tiles = gr.hi - gr.lo; rg.isect_lo = gr.base;
            return rg;
        };
        // one run's launch: its tiles, its K, its slice of the chunk buffers
        long long chunk_off = 0;
        std::vector<RasterArgs> run_args;
        for (const RasterRun &r : runs) {
            RasterArgs rr = ra;
            rr.tile_lo = vt.tile_base[r.v0];
            rr.num_tiles = vt.tile_base[r.v1] - vt.tile_base[r.v0];
            rr.k_max = r.k;
            rr.chunk_p0 = vt.pix_base[r.v0];
            rr.chunk_P = vt.pix_base[r.v1] - vt.pix_base[r.v0];
            if (r.k > 1) {
                rr.chunk_T = ptr<float>("chunk_T") + chunk_off; rr.chunk_C = ptr<float>("chunk_C") + 3 * chunk_off;
                rr.chunk_idx = ptr<int>("chunk_idx") + chunk_off;
                rr.prefix_T = ptr<float>("prefix_T") + chunk_off; rr.after_C = ptr<float>("after_C") + 3 * chunk_off;
                chunk_off += (long long)r.k * rr.chunk_P;
            }
            run_args.push_back(rr);
        }
        if (!fixed) {
            for (const RasterArgs &rr : run_args) launch_raster_fwd(rr, stream_);
        } else {
            for (const TileGroup &gr : groups) {
                build_group(gr);
                launch_raster_fwd(group_raster(gr), stream_);
            }
            launches_ += (long long)groups.size() - 1;
        }
        debug_sync(stream_, "raster_fwd");
        last_ra_ = fixed ? ra : run_args[0];   // (backward_image: one view, one run)
        mark(3);
        if (!has_gt) { mark(4); mark(5); mark(6); mark(7); mark(8); return; }

        LossArgs la{};
        la.vt = vt; la.sp = pa.sp; la.img = ra.out_img;
        la.gt = nullptr; la.mask = nullptr;   // read from StepParams (see common.cuh)
        la.v_img = ptr<float>("v_img");
        la.loss_sum = ptr<float>("loss_sum"); la.nan_counts = pa.nan_counts;
        const int nl = launch_loss(la, stream_);
        if (nl < 0) throw std::runtime_error("loss kernel set-up failed");
        launches_ += nl;
        debug_sync(stream_, "loss");
        mark(4);
        if (!backward) { mark(5); mark(6); mark(7); mark(8); return; }

        if (!fixed) {
            for (const RasterArgs &rr : run_args) launch_raster_bwd(rr, stream_);
        } else {
            // one group: its lists are still in the buffer; several: each
            // group's lists are rebuilt (the same sorted order) for its backward
            for (const TileGroup &gr : groups) {
                if (groups.size() > 1) build_group(gr);
                launch_raster_bwd(group_raster(gr), stream_);
            }
            launches_ += (long long)groups.size() - 1;
        }
        debug_sync(stream_, "raster_bwd");
        mark(5);

        ProjectBwdArgs pb{};
        pb.vt = vt; pb.rest_bases = g.rest_bases; pb.do_optimizer = opt;
        pb.sp = pa.sp;
        pb.means = g.means; pb.scales = g.scales; pb.quats = g.quats; pb.radii = pa.radii; pb.rec = pa.rec;
        pb.grad = ra.grad;
        pb.v_mean = ptr<float>("v_mean"); pb.v_scale = ptr<float>("v_scale"); pb.v_quat = ptr<float>("v_quat");
        pb.v_opac = B > 1 ? ptr<float>("v_opac") : nullptr;
        pb.sh_in = ptr<float4>("sh_in");
        pb.features_dc = g.features_dc; pb.features_rest = g.features_rest;
        if (st) {
            pb.dc_m = st->exp_avg[3]; pb.dc_v = st->exp_avg_sq[3];
            pb.rest_m = st->exp_avg[4]; pb.rest_v = st->exp_avg_sq[4];
        }
        pb.nan_counts = pa.nan_counts;
        pb.gstats = gstats_;
        launch_project_bwd(pb, stream_);
        debug_sync(stream_, "project_bwd");
        mark(6);

        AdamArgs aa{};
        aa.n = N; aa.sp = pa.sp;
        aa.means = g.means; aa.scales = g.scales; aa.quats = g.quats; aa.opacities = g.opacities;
        if (st) {
            const int grp[4] = {0, 1, 2, 5};
            for (int k = 0; k < 4; k++) { aa.m[k] = st->exp_avg[grp[k]]; aa.v[k] = st->exp_avg_sq[grp[k]]; }
            aa.dc_v = st->exp_avg_sq[3];
        }
        aa.g_mean = pb.v_mean; aa.g_scale = pb.v_scale; aa.g_quat = pb.v_quat; aa.grad = ra.grad;
        aa.g_opac = pb.v_opac;
        aa.nan_counts = pa.nan_counts;
        if (opt) launch_adam(aa, num_sms_, stream_);
        debug_sync(stream_, "adam");
        mark(7);
        if (a0.do_sgld) launch_sgld(aa, stream_);
        debug_sync(stream_, "sgld");
        mark(8);
        CK(cudaGetLastError());
        };   // issue

        // CUDA graph mode: the second step with the same shapes and buffers
        // is captured, later ones replay it (one launch for the whole step).
        // The targets and masks come through StepParams, not the key.
        const bool graphable = use_graphs_ && !timing_ && !g_sync_check && !fixed;
        if (graphable) {
            std::string ks;
            auto put = [&](const void *p, size_t n) { ks.append(reinterpret_cast<const char *>(p), n); };
            const int head[4] = {N, B, g.rest_bases,
                                 (a0.do_optimizer ? 1 : 0) | (a0.do_sgld ? 2 : 0) | (backward ? 4 : 0) | (st ? 8 : 0) |
                                     (has_gt ? 16 : 0)};
            put(head, sizeof(head));
            put(Kv, sizeof(int) * B);
            put(&tune, sizeof(tune));
            put(w, sizeof(int) * B);
            put(h, sizeof(int) * B);
            const void *ps[20] = {g.means, g.scales, g.quats, g.features_dc, g.features_rest, g.opacities, gstats_};
            for (int k = 0; k < 6 && st; k++) { ps[8 + k] = st->exp_avg[k]; ps[14 + k] = st->exp_avg_sq[k]; }
            put(ps, sizeof(ps));
            auto it = graphs_.find(ks);
            if (it != graphs_.end()) {
                CK(cudaGraphLaunch(it->second.exec, stream_));
                launches_ += it->second.launches;
                return;
            }
            if (graph_seen_.count(ks) && graphs_.size() < kMaxGraphs) {
                const long long l0 = launches_;
                cudaGraph_t graph = nullptr;
                CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
                try {
                    issue();
                } catch (...) {
                    cudaStreamEndCapture(stream_, &graph);
                    if (graph) cudaGraphDestroy(graph);
                    throw;
                }
                CK(cudaStreamEndCapture(stream_, &graph));
                cudaGraphExec_t exec = nullptr;
                const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                CK(ie);
                graphs_[ks] = GraphEntry{exec, launches_ - l0};
                CK(cudaGraphLaunch(exec, stream_));
                return;
            }
            graph_seen_.insert(ks);
        }
        issue();
    }

  public:
    // dL/d(parameters) for a caller-supplied dL/d(image): the forward is run
    // again (projection, tile lists, raster) rather than kept from an
    // earlier call, then the raster and projection backward passes write
    // the gradients into the caller's buffers.  No optimizer step.
    void backward_image(const MsplatGaussians &g, const MsplatStepArgs &args, const float *v_img,
                        const MsplatGradients &out) {
        if (!v_img) throw std::runtime_error("v_img is null");
        if (!out.v_means || !out.v_scales || !out.v_quats || !out.v_opacities || !out.v_features_dc ||
            (g.rest_bases > 0 && !out.v_features_rest))
            throw std::runtime_error("null gradient pointer");
        // The raster arguments of this forward are needed below for the whole
        // view at once: a fixed intersection budget is used when the view's
        // lists fit it in one group (an error otherwise), else the legacy
        // per-view buffer.
        const bool graphs = use_graphs_;
        use_graphs_ = false;
        try {
            train_step(g, nullptr, args, nullptr, nullptr, false);
        } catch (...) {
            use_graphs_ = graphs;
            throw;
        }
        use_graphs_ = graphs;
        if (last_groups_ > 1)
            throw std::runtime_error("backward: the view's intersections need " + std::to_string(last_groups_) +
                                     " tile groups under the intersection budget; the backward takes one");
        const int N = g.num_points;
        if (N <= 0) return;
        CK(cudaMemsetAsync(ptr<GradRec>("grad"), 0, sizeof(GradRec) * (size_t)N, stream_));
        RasterArgs ra = last_ra_;   // one view
        ra.v_img = v_img;
        ra.grad = ptr<GradRec>("grad");
        launch_raster_bwd(ra, stream_);
        debug_sync(stream_, "raster_bwd");
        ProjectBwdArgs pb{};
        pb.vt = ra.vt; pb.rest_bases = g.rest_bases; pb.do_optimizer = 0;
        pb.sp = ptr<StepParams>("params");
        pb.means = g.means; pb.scales = g.scales; pb.quats = g.quats;
        pb.radii = ptr<int>("radii"); pb.rec = ptr<SplatRec>("rec"); pb.grad = ra.grad;
        pb.v_mean = out.v_means; pb.v_scale = out.v_scales; pb.v_quat = out.v_quats;
        pb.features_dc = g.features_dc; pb.features_rest = g.features_rest;
        pb.v_dc_out = out.v_features_dc; pb.v_rest_out = out.v_features_rest; pb.v_opac_out = out.v_opacities;
        pb.sh_in = ptr<float4>("sh_in");
        pb.nan_counts = ptr<unsigned>("nan_counts");
        launch_project_bwd(pb, stream_);
        debug_sync(stream_, "project_bwd");
        launches_ += (last_K_ > 1 ? 2 : 1) + 2;
        CK(cudaGetLastError());
    }

    void set_isect_budget(long long slots) {
        if (slots < 0) throw std::runtime_error("negative intersection budget");
        if (slots >= (1LL << 31)) throw std::runtime_error("intersection budget of 2^31 slots or more");
        if (slots != isect_slots_) clear_graphs();
        isect_slots_ = slots;
    }

    void set_tuning(const MsplatTuning &t) {
        if (t.sort_width != 256 && t.sort_width != 512) throw std::runtime_error("sort_width must be 256 or 512");
        if (t.raster_batch != 128 && t.raster_batch != 256) throw std::runtime_error("raster_batch must be 128 or 256");
        if (t.chunk != 256 && t.chunk != 512 && t.chunk != 1024) throw std::runtime_error("chunk must be 256, 512 or 1024");
        if (t.raster_mode < 0 || t.raster_mode > 2) throw std::runtime_error("raster_mode must be 0, 1 or 2");
        if (t.tile_order < 0 || t.tile_order > 1) throw std::runtime_error("tile_order must be 0 or 1");
        if (t.tile_split != 1 && t.tile_split != 2) throw std::runtime_error("tile_split must be 1 or 2");
        if (t.bwd_pixels != 1 && t.bwd_pixels != 2) throw std::runtime_error("bwd_pixels must be 1 or 2");
        if (std::memcmp(&t, &tuning_, sizeof(t)) != 0) clear_graphs();
        tuning_ = t;
    }
    MsplatTuning tuning() const { return tuning_; }

    // Coordinate-wise search over the tunable launch configuration, timing
    // whole steps (no optimizer, no SGLD, no activity statistics) eagerly.
    MsplatTuning autotune(const MsplatGaussians &g, const MsplatStepArgs *args, int B, const uint8_t *const *gts,
                          const uint8_t *const *masks, int reps, float *best_ms) {
        if (B <= 0 || B > kMaxViews) throw std::runtime_error("autotune: 1 to 16 views");
        for (int v = 0; v < B; v++)
            if (!gts || !gts[v]) throw std::runtime_error("autotune: a target image per view is needed");
        reps = std::max(1, std::min(reps, 50));
        std::vector<MsplatStepArgs> a(args, args + B);
        for (auto &x : a) { x.do_optimizer = 0; x.do_sgld = 0; }
        float4 *gs = gstats_;
        const bool graphs = use_graphs_, timing = timing_;
        gstats_ = nullptr;
        use_graphs_ = false;
        timing_ = false;
        const MsplatTuning start = tuning_;
        auto measure = [&](const MsplatTuning &t) {
            tuning_ = t;
            run_views(g, nullptr, a.data(), B, gts, masks, true);   // warm-up (and buffer growth)
            std::vector<float> ms(reps);
            for (int r = 0; r < reps; r++) {
                CK(cudaEventRecord(marker_[0], stream_));
                run_views(g, nullptr, a.data(), B, gts, masks, true);
                CK(cudaEventRecord(marker_[1], stream_));
                CK(cudaEventSynchronize(marker_[1]));
                CK(cudaEventElapsedTime(&ms[r], marker_[0], marker_[1]));
            }
            std::sort(ms.begin(), ms.end());
            return ms[reps / 2];
        };
        MsplatTuning best = start;
        float bms = 0.f;
        try {
            // untimed steps first, so the clocks have ramped up before the
            // starting configuration is timed; a candidate replaces the best
            // only when it is faster by more than 1 % (timing noise)
            for (int r = 0; r < 10; r++) run_views(g, nullptr, a.data(), B, gts, masks, true);
            bms = measure(best);
            auto consider = [&](MsplatTuning c) {
                if (std::memcmp(&c, &best, sizeof(c)) == 0) return;
                const float m = measure(c);
                if (m < 0.99f * bms) { bms = m; best = c; }
            };
            for (int o : {0, 1}) { MsplatTuning c = best; c.tile_order = o; consider(c); }
            for (int w : {256, 512}) { MsplatTuning c = best; c.sort_width = w; consider(c); }
            for (int p : {1, 2}) { MsplatTuning c = best; c.tile_split = p; consider(c); }
            for (int b : {128, 256}) { MsplatTuning c = best; c.raster_batch = b; consider(c); }
            for (int p : {1, 2}) { MsplatTuning c = best; c.bwd_pixels = p; consider(c); }
            if (a[0].raster_mode == 0) {
                { MsplatTuning c = best; c.raster_mode = 1; consider(c); }
                for (int ch : {256, 512, 1024}) { MsplatTuning c = best; c.raster_mode = 2; c.chunk = ch; consider(c); }
            }
        } catch (...) {
            tuning_ = start;
            gstats_ = gs;
            use_graphs_ = graphs;
            timing_ = timing;
            throw;
        }
        gstats_ = gs;
        use_graphs_ = graphs;
        timing_ = timing;
        tuning_ = best;
        clear_graphs();
        if (best_ms) *best_ms = bms;
        return best;
    }

    void mcmc(const MsplatGaussians &g, const MsplatAdamState &st, int cap_max, float cull_radius,
              int &relocation_count, MsplatMcmcStats &out, const float *score = nullptr) {
        CK(cudaSetDevice(device_));
        if (cap_max < g.num_points) throw std::runtime_error("cap_max below the active count");
        const size_t cap = (size_t)std::max(cap_max, 1);
        const size_t parts = cap / 2048 + 2;
        alloc("mcmc_flags", cap * 4);
        alloc("mcmc_pos", cap * 4);
        alloc("mcmc_copies", cap * 4);
        alloc("mcmc_weights", cap * 8);
        alloc("mcmc_cumw", cap * 8);
        alloc("mcmc_upart", parts * 4);
        alloc("mcmc_dpart", parts * 8);
        alloc("mcmc_dead", cap * 4);
        alloc("mcmc_moves", cap * 16);
        alloc("mcmc_counters", 64, true);
        McmcArgs a{};
        a.n = g.num_points; a.rest_bases = g.rest_bases;
        a.means = g.means; a.scales = g.scales; a.quats = g.quats; a.features_dc = g.features_dc;
        a.features_rest = g.features_rest; a.opacities = g.opacities;
        for (int k = 0; k < 6; k++) { a.exp_avg[k] = st.exp_avg[k]; a.exp_avg_sq[k] = st.exp_avg_sq[k]; }
        a.cull_r2 = cull_radius > 0.f ? cull_radius * cull_radius : -1.f;
        a.flags = ptr<uint32_t>("mcmc_flags"); a.flag_pos = ptr<uint32_t>("mcmc_pos");
        a.upart = ptr<uint32_t>("mcmc_upart"); a.copies = ptr<uint32_t>("mcmc_copies");
        a.weights = ptr<double>("mcmc_weights"); a.cumw = ptr<double>("mcmc_cumw"); a.dpart = ptr<double>("mcmc_dpart");
        a.dead_list = ptr<int>("mcmc_dead"); a.moves = ptr<int>("mcmc_moves");
        a.counters = ptr<unsigned>("mcmc_counters");
        a.score = score;
        a.gstats = gstats_;
        McmcResult r;
        run_mcmc(a, cap_max, relocation_count, r, stream_);
        out.num_dead = r.num_dead; out.num_culled = r.num_culled; out.num_nonfinite = r.num_nonfinite;
        out.num_relocated = r.num_relocated; out.num_grown = r.num_grown; out.num_active = r.num_active;
    }

    void synchronize() { CK(cudaStreamSynchronize(stream_)); }

    float loss() {
        float v[kMaxViews] = {0.f};
        const int B = std::max(1, last_views_);
        CK(cudaMemcpyAsync(v, ptr<float>("loss_sum"), sizeof(float) * B, cudaMemcpyDeviceToHost, stream_));
        synchronize();
        if (B == 1) return v[0] / (float)last_view_P_[0];
        double acc = 0;   // several views: the mean of the views' losses
        for (int k = 0; k < B; k++) acc += (double)v[k] / (double)last_view_P_[k];
        return (float)(acc / (double)B);
    }

    void stats(MsplatEngineStats &o) {
        std::memset(&o, 0, sizeof(o));
        synchronize();
        if (last_T_ > 0) {
            uint32_t tot = 0, mx = 0;
            CK(cudaMemcpy(&tot, ptr<uint32_t>("tile_offsets") + last_T_, 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(&mx, ptr<uint32_t>("max_tile"), 4, cudaMemcpyDeviceToHost));
            o.num_intersections = tot;
            o.max_tile_count = (int)mx;
        }
        o.k_max = last_K_;
        o.num_tiles = last_T_;
        o.isect_groups = last_groups_;
        if (has("nan_counts")) {
            unsigned tmp[32];
            CK(cudaMemcpy(tmp, ptr<unsigned>("nan_counts"), sizeof(tmp), cudaMemcpyDeviceToHost));
            std::memcpy(o.nan_counts, tmp, 64);
            std::memcpy(o.check_record, tmp + kDbgSlot, sizeof(o.check_record));
        }
        o.launches = launches_;
        o.timed_steps = timed_steps_;
        // stage time summed over the timed steps still held in the ring
        const long long held = std::min<long long>(timed_steps_, kRing);
        for (long long r = 0; r < held; r++)
            for (int s = 0; s < MSPLAT_STAGE_COUNT; s++) {
                float ms = 0;
                if (cudaEventElapsedTime(&ms, ev_[r][s], ev_[r][s + 1]) == cudaSuccess) o.stage_ms[s] += ms;
            }
        o.timed_steps = held;
    }

    void record_marker(int which) { CK(cudaEventRecord(marker_[which & 1], stream_)); }
    float marker_elapsed() {
        CK(cudaEventSynchronize(marker_[1]));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, marker_[0], marker_[1]));
        return ms;
    }

    void set_timing(bool on) {
        timing_ = on;
        timed_steps_ = 0;
    }

    long long buffer(const std::string &name, void **p) {
        auto it = bufs_.find(name);
        if (it == bufs_.end()) return -1;
        if (p) *p = it->second.ptr;
        return (long long)it->second.bytes;
    }

    cudaStream_t stream() const { return stream_; }
    std::string err;

  private:
    template <class T> T *ptr(const char *name) { return reinterpret_cast<T *>(bufs_.at(name).ptr); }
    bool has(const char *name) const { return bufs_.count(name) > 0; }

    void alloc(const char *name, size_t bytes, bool zero = false) {
        Buf &b = bufs_[name];
        if (b.bytes >= bytes && b.ptr) return;
        if (b.ptr) {
            CK(cudaStreamSynchronize(stream_));
            CK(cudaFree(b.ptr));
            clear_graphs();   // captured steps hold the old address
        }
        b.ptr = nullptr;
        CK(cudaMalloc(&b.ptr, std::max<size_t>(bytes, 256)));
        b.bytes = bytes;
        if (zero) CK(cudaMemsetAsync(b.ptr, 0, bytes, stream_));
    }

    // per-record buffers for `views` x n records, per-Gaussian gradients for n
    void ensure_points(int n, int views = 1) {
        if (!has("params")) {
            alloc("params", sizeof(StepParams) * kMaxViews);
            alloc("loss_sum", 256, true);
            alloc("nan_counts", 128, true);
            alloc("max_tile", 256, true);
        }
        const long long recs = (long long)n * views;
        if (recs > cap_records_ || !has("rec")) {
            const size_t m = (size_t)std::max<long long>(recs, 1);
            alloc("rec", m * sizeof(SplatRec));
            alloc("depths", m * 4);
            alloc("radii", m * 4);
            alloc("aabb", m * 8);
            alloc("tiles_hit", m * 4);
            alloc("grad", m * sizeof(GradRec), true);
            cap_records_ = recs;
        }
        if (n > cap_points_ || !has("v_mean")) {
            const size_t m = (size_t)std::max(n, 1);
            alloc("v_mean", m * 12);
            alloc("v_scale", m * 12);
            alloc("v_quat", m * 16);
            alloc("v_opac", m * 4);
            alloc("sh_in", m * 16);
            cap_points_ = n;
        }
    }
    void ensure_tiles(int T) {
        if (T <= cap_tiles_) return;
        alloc("tile_counts", (size_t)2 * T * 4);
        alloc("tile_offsets", (size_t)(T + 1) * 4);
        alloc("tile_lists", (size_t)4 * T * 4);
        alloc("tile_class", 64, true);
        cap_tiles_ = T;
    }
    void ensure_isect(long long c) {
        if (c <= cap_isect_) return;
        alloc("keys", (size_t)c * 8);
        alloc("keys_alt", (size_t)c * 8);
        alloc("isect_ids", (size_t)c * 4);
        cap_isect_ = c;
    }
    void ensure_pixels(long long P) {
        if (P <= cap_pixels_) return;
        alloc("out_img", (size_t)P * 12);
        alloc("final_T", (size_t)P * 4);
        alloc("final_idx", (size_t)P * 4);
        alloc("v_img", (size_t)P * 12);
        cap_pixels_ = P;
    }
    void ensure_chunks(long long KP) {
        if (KP <= cap_chunks_) return;
        alloc("chunk_T", (size_t)KP * 4);
        alloc("chunk_C", (size_t)KP * 12);
        alloc("chunk_idx", (size_t)KP * 4);
        alloc("prefix_T", (size_t)KP * 4);
        alloc("after_C", (size_t)KP * 12);
        cap_chunks_ = KP;
    }

    // Consecutive tiles whose intersections fit `slots` (isect_tile_groups,
    // msplat_metal.mm:693-718, with exact rather than padded bucket sizes).
    struct TileGroup {
        int lo, hi;
        long long base;   // global slot of the group's first intersection
    };
    static std::vector<TileGroup> tile_groups(const std::vector<uint32_t> &counts, long long slots) {
        std::vector<TileGroup> groups;
        long long used = 0, base = 0;
        int lo = 0;
        for (int t = 0; t < (int)counts.size(); t++) {
            const long long c = counts[t];
            if (c == 0) continue;
            if (c > slots)
                throw std::runtime_error("tile " + std::to_string(t) + " has " + std::to_string(c) +
                                         " intersections, more than the fixed budget's " + std::to_string(slots));
            if (used + c > slots) {
                groups.push_back({lo, t, base});
                lo = t;
                base += used;
                used = 0;
            }
            used += c;
        }
        groups.push_back({lo, (int)counts.size(), base});
        return groups;
    }

    // Maximal runs of consecutive views with the same depth-chunk count:
    // one raster launch (and merge / prefix-suffix) per run, so a batch of
    // equal views is one launch per stage.
    struct RasterRun {
        int v0, v1, k;   // views [v0, v1), chunks per tile (1: monolithic)
    };
    static std::vector<RasterRun> raster_runs(const ViewTable &vt, const int *Kv) {
        std::vector<RasterRun> runs;
        for (int v = 0; v < vt.count; v++) {
            if (!runs.empty() && runs.back().k == Kv[v]) runs.back().v1 = v + 1;
            else runs.push_back({v, v + 1, Kv[v]});
        }
        return runs;
    }

    // K_max rule, msplat_metal.mm:1204-1224; a step in auto mode takes the
    // tuned mode, and the chunk length is the tuned one (the reference's 512
    // by default)
    static int choose_k(const MsplatStepArgs &a, int T, long long cap, const MsplatTuning &t) {
        const int mode = a.raster_mode != 0 ? a.raster_mode : t.raster_mode;
        if (mode == 1) return 1;
        if (mode == 0 && T >= 400) return 1;
        if (a.k_max > 0) return a.k_max;
        const uint32_t chunk = (uint32_t)t.chunk;
        const uint32_t avg = (uint32_t)(cap / std::max(1, T));
        const uint32_t cons = avg * 6;
        uint32_t k = (cons + chunk - 1) / chunk;
        if (k < 2) k = 2;
        const uint32_t am = (uint32_t)((cap + chunk - 1) / chunk);
        if (k > am) k = am;
        return (int)k;
    }

    static void fill_params(const MsplatStepArgs &a, StepParams &sp, bool has_mask) {
        std::memset(&sp, 0, sizeof(sp));
        std::memcpy(sp.viewmat, a.viewmat, sizeof(sp.viewmat));
        std::memcpy(sp.projmat, a.projmat, sizeof(sp.projmat));
        sp.fx = a.fx; sp.fy = a.fy; sp.cx = a.cx; sp.cy = a.cy;
        sp.tan_fovx = 0.5f * (float)a.width / a.fx;    // msplat_metal.metal:1771
        sp.tan_fovy = 0.5f * (float)a.height / a.fy;
        std::memcpy(sp.cam_pos, a.cam_pos, sizeof(sp.cam_pos));
        std::memcpy(sp.bg, a.background, sizeof(sp.bg));
        sp.clip_thresh = a.clip_thresh;
        sp.degrees_to_use = a.degrees_to_use;
        sp.ssim_weight = a.ssim_weight;
        sp.loss_inv_n = a.loss_inv_n;
        std::memcpy(sp.step_size, a.step_size, sizeof(sp.step_size));
        std::memcpy(sp.bc2_sqrt, a.bc2_sqrt, sizeof(sp.bc2_sqrt));
        sp.beta1 = a.beta1; sp.beta2 = a.beta2; sp.eps = a.eps;
        sp.op_reg = a.op_reg; sp.sc_reg = a.sc_reg; sp.invis_scale = a.invis_scale;
        sp.seed = a.seed; sp.noise_lr = a.noise_lr; sp.xyz_lr = a.xyz_lr; sp.max_disp = a.max_disp;
        sp.has_mask = has_mask ? 1 : 0;
    }

    static void validate(const MsplatGaussians &g, const MsplatStepArgs &a) {
        if (g.num_points < 0) throw std::runtime_error("num_points < 0");
        if (a.width <= 0 || a.height <= 0) throw std::runtime_error("image size must be positive");
        if ((long long)a.width * a.height > (1LL << 31) / 16) throw std::runtime_error("image too large");
        if (g.rest_bases < 0 || g.rest_bases > 15) throw std::runtime_error("rest_bases must be in [0, 15]");
        if (g.num_points > 0 && (!g.means || !g.scales || !g.quats || !g.features_dc || !g.opacities ||
                                 (g.rest_bases > 0 && !g.features_rest)))
            throw std::runtime_error("null parameter pointer");
        if (g.num_points > (1 << 26)) throw std::runtime_error("more than 2^26 Gaussians");
        if (((uintptr_t)g.quats & 15) != 0) throw std::runtime_error("quats must be 16-byte aligned");
    }

    void mark(int s) {
        if (timing_) CK(cudaEventRecord(ev_[slot_][s], stream_));
    }

    int device_ = 0, num_sms_ = 1;
    cudaStream_t stream_ = nullptr;
    cudaStream_t copy_stream_ = nullptr;          // host-image uploads
    cudaEvent_t stage_ready_[2], stage_free_[2];  // per stage buffer: upload done / last reader done
    int stage_slot_ = 0;
    std::map<std::string, Buf> bufs_;
    int cap_points_ = 0, cap_tiles_ = 0;
    long long cap_records_ = 0, cap_isect_ = 0, cap_pixels_ = 0, cap_chunks_ = 0;
    int last_T_ = 0, last_K_ = 1, last_views_ = 1;
    long long last_view_P_[kMaxViews] = {1};   // pixels of each view of the last step
    bool timing_ = false;
    static constexpr int kRing = 128;
    cudaEvent_t ev_[kRing][MSPLAT_STAGE_COUNT + 1];
    cudaEvent_t marker_[2];
    int slot_ = 0;
    long long timed_steps_ = 0, launches_ = 0;
    RasterArgs last_ra_{};   // raster arguments of the last eagerly issued step
    float4 *gstats_ = nullptr;   // caller's activity statistics (learned relocation), or null
    MsplatTuning tuning_{512, 128, kChunk, 0, 1, 1, 2};   // launch configuration of the tunable stages
    long long isect_slots_ = 0;   // fixed intersection budget in slots (0: legacy 48 per Gaussian and view)
    int last_groups_ = 1;         // tile groups of the last step

  public:
    void set_gstats(void *p) { gstats_ = static_cast<float4 *>(p); }

  private:

    // captured steps, keyed by shapes, flags and every pointer they bake in
    struct GraphEntry {
        cudaGraphExec_t exec;
        long long launches;
    };
    static constexpr size_t kMaxGraphs = 512;
    bool use_graphs_ = false;
    std::map<std::string, GraphEntry> graphs_;
    std::set<std::string> graph_seen_;

  public:
    void set_graphs(bool on) {
        use_graphs_ = on;
        if (!on) clear_graphs();
    }
    void clear_graphs() {
        for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second.exec);
        graphs_.clear();
        graph_seen_.clear();
    }
};

}  // namespace msplat

struct MsplatEngine {
    msplat::Engine *impl = nullptr;
    std::string err;
};

template <class F> static int guarded(MsplatEngine *e, F &&f) {
    if (!e || !e->impl) return -1;
    try {
        f();
        return 0;
    } catch (const std::exception &ex) {
        e->err = ex.what();
        fprintf(stderr, "msplat engine: %s\n", ex.what());
        return -2;
    }
}

extern "C" {

MsplatEngine *msplat_engine_create(int device, int max_points) {
    auto *e = new MsplatEngine();
    try {
        e->impl = new msplat::Engine(device);
        if (max_points > 0) e->impl->reserve_points(max_points);
    } catch (const std::exception &ex) {
        fprintf(stderr, "msplat engine: %s\n", ex.what());
        delete e->impl;
        delete e;
        return nullptr;
    }
    return e;
}

void msplat_engine_destroy(MsplatEngine *e) {
    if (!e) return;
    delete e->impl;
    delete e;
}

const char *msplat_engine_last_error(const MsplatEngine *e) { return e ? e->err.c_str() : "null engine"; }

int msplat_engine_train_step(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st,
                             const MsplatStepArgs *args, const uint8_t *gt, const uint8_t *mask) {
    if (!g || !args || !gt) return -1;
    return guarded(e, [&] { e->impl->train_step(*g, st, *args, gt, mask, true); });
}

int msplat_engine_train_step_host(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st,
                                  const MsplatStepArgs *args, const uint8_t *gt_host, const uint8_t *mask_host) {
    if (!g || !args || !gt_host) return -1;
    return guarded(e, [&] { e->impl->train_step_host(*g, st, *args, gt_host, mask_host); });
}

int msplat_engine_render(MsplatEngine *e, const MsplatGaussians *g, const MsplatStepArgs *args) {
    if (!g || !args) return -1;
    return guarded(e, [&] { e->impl->train_step(*g, nullptr, *args, nullptr, nullptr, false); });
}

int msplat_engine_synchronize(MsplatEngine *e) {
    return guarded(e, [&] { e->impl->synchronize(); });
}

int msplat_engine_loss_async(MsplatEngine *e, float *dst) {
    if (!dst) return -1;
    return guarded(e, [&] { e->impl->loss_async(dst); });
}

int msplat_engine_loss(MsplatEngine *e, float *loss) {
    if (!loss) return -1;
    return guarded(e, [&] { *loss = e->impl->loss(); });
}

int msplat_engine_stats(MsplatEngine *e, MsplatEngineStats *out) {
    if (!out) return -1;
    return guarded(e, [&] { e->impl->stats(*out); });
}

int msplat_engine_set_timing(MsplatEngine *e, int enabled) {
    return guarded(e, [&] { e->impl->set_timing(enabled != 0); });
}

long long msplat_engine_buffer(MsplatEngine *e, const char *name, void **dev_ptr) {
    if (!e || !e->impl || !name) return -1;
    return e->impl->buffer(name, dev_ptr);
}

int msplat_engine_read(MsplatEngine *e, const char *name, void *dst, long long bytes) {
    if (!e || !e->impl || !name || !dst) return -1;
    return guarded(e, [&] {
        void *p = nullptr;
        const long long have = e->impl->buffer(name, &p);
        if (have < 0) throw std::runtime_error(std::string("no buffer ") + name);
        if (bytes > have) throw std::runtime_error(std::string("read past the end of ") + name);
        // on the engine's stream, host or device destination; done on return
        CK(cudaMemcpyAsync(dst, p, (size_t)bytes, cudaMemcpyDefault, e->impl->stream()));
        e->impl->synchronize();
    });
}

int msplat_engine_mcmc(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st, int cap_max,
                       float cull_radius, int *relocation_count, MsplatMcmcStats *out) {
    if (!g || !st || !relocation_count || !out) return -1;
    return guarded(e, [&] { e->impl->mcmc(*g, *st, cap_max, cull_radius, *relocation_count, *out); });
}

int msplat_engine_backward(MsplatEngine *e, const MsplatGaussians *g, const MsplatStepArgs *args, const float *v_img,
                           const MsplatGradients *out) {
    if (!g || !args || !out) return -1;
    return guarded(e, [&] { e->impl->backward_image(*g, *args, v_img, *out); });
}

int msplat_engine_train_step_batch(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st,
                                   const MsplatStepArgs *args, int num_views, const uint8_t *const *gt,
                                   const uint8_t *const *mask) {
    if (!g || !st || !args || !gt || num_views <= 0) return -1;
    return guarded(e, [&] { e->impl->train_step_batch(*g, *st, args, num_views, gt, mask); });
}

int msplat_engine_set_activity_stats(MsplatEngine *e, void *stats) {
    return guarded(e, [&] { e->impl->set_gstats(stats); });
}

int msplat_engine_mcmc_scored(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st, int cap_max,
                              float cull_radius, int *relocation_count, const float *score, MsplatMcmcStats *out) {
    if (!g || !st || !relocation_count || !out) return -1;
    return guarded(e, [&] { e->impl->mcmc(*g, *st, cap_max, cull_radius, *relocation_count, *out, score); });
}

int msplat_engine_set_isect_budget(MsplatEngine *e, long long slots) {
    return guarded(e, [&] { e->impl->set_isect_budget(slots); });
}

int msplat_engine_set_tuning(MsplatEngine *e, const MsplatTuning *t) {
    if (!t) return -1;
    return guarded(e, [&] { e->impl->set_tuning(*t); });
}

int msplat_engine_get_tuning(MsplatEngine *e, MsplatTuning *t) {
    if (!t) return -1;
    return guarded(e, [&] { *t = e->impl->tuning(); });
}

int msplat_engine_autotune(MsplatEngine *e, const MsplatGaussians *g, const MsplatStepArgs *args, int num_views,
                           const uint8_t *const *gt, const uint8_t *const *mask, int reps, MsplatTuning *out,
                           float *ms) {
    if (!g || !args || !out) return -1;
    return guarded(e, [&] { *out = e->impl->autotune(*g, args, num_views, gt, mask, reps, ms); });
}

int msplat_engine_set_graphs(MsplatEngine *e, int enabled) {
    return guarded(e, [&] { e->impl->set_graphs(enabled != 0); });
}

int msplat_engine_marker(MsplatEngine *e, int which) {
    return guarded(e, [&] { e->impl->record_marker(which); });
}

int msplat_engine_marker_elapsed(MsplatEngine *e, float *ms) {
    if (!ms) return -1;
    return guarded(e, [&] { *ms = e->impl->marker_elapsed(); });
}

void *msplat_engine_stream(MsplatEngine *e) { return (e && e->impl) ? (void *)e->impl->stream() : nullptr; }

}  // extern "C"
