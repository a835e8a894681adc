// server.cu — serving loop: many camera streams, continuous batching.
//
// A server owns frame slots in one arena, grouped by frame size class and
// sized from an HBM budget (admission: a frame is accepted only when a slot
// of its size is free).  Each stream keeps its keyframe's features resident
// in a slot and every incoming frame is matched against it; a frame can
// promote itself to the stream's keyframe (the stream's first frame always
// does) -- the device-side counterpart of FeatureSet(1) advancing in
// LoadDataCPUPass::shiftFeatureSets (load_features_cpu.cpp:111-142).
//
// A dispatcher thread launches, whenever requests are waiting and fewer than
// two launches are in flight, one batch of everything queued (up to
// max_batch frames): H2D of the frames from pinned staging, its work tables,
// and the kernels of the batch path over those frames and their
// (keyframe, frame) pairs.  Launches alternate between two CUDA streams, so
// a batch admitted while another is on the GPU runs alongside it; a pair
// whose keyframe is produced by a launch still in flight on the other stream
// waits for that launch's event.  Results are bit-identical to the batch
// path: the kernels are the same and no kernel reads another frame's data
// except its pair's keyframe.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "runtime_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct SrvClass {
    int W0 = 0, H0 = 0;
    int first_slot = 0, n_slots = 0;
    int tiles_per_frame = 0;
    int shape = 0;                // detect tile shape (index into kTileShapes)
    std::vector<TileItem> tiles;  // one frame's tile list (frame field patched per launch)
    std::vector<BandItem> bands;  // one frame's compaction bands (frame field patched per launch)
    std::vector<BandItem> desc;   // one frame's describe items (chunks of the bands)
};

struct SrvSlot {
    int cls = 0;
    bool in_use = false;       // owned by a request (until released)
    bool keyframe = false;     // held by a stream as its keyframe
    int refs = 0;              // requests queued or in flight that match against it
    int producer_launch = -1;  // in-flight launch that writes its features, or -1
    uint8_t* h_in = nullptr;   // pinned staging of the frame
    int32_t* a2b = nullptr;    // pair scratch when this slot is the current frame
    uint4* bacc = nullptr;     // k_match's b -> a accumulators when this slot is the current frame
    int32_t* matches = nullptr;
    uint32_t* match_count = nullptr;
    uint32_t* h_res = nullptr;  // pinned, mapped: the frame's results as the emit kernel lays them out
    uint32_t* d_res = nullptr;  // device address of h_res
};

struct SrvReq {
    int stream = 0, slot = 0, ref = -1;
    bool promote = false, done = false;
    bool failed = false;  // finished without results (a failed launch, or queued at a failure)
    Clock::time_point t_submit, t_done;
};

struct SrvStream {
    int cls = 0;
    int keyframe = -1;
};

struct SrvLaunch {
    int id = 0;
    int buf = 0;
    cudaEvent_t done = nullptr;
    std::vector<uint64_t> tickets;
};

struct LaunchBuf {
    char* h = nullptr;  // pinned table image
    char* d = nullptr;  // device tables
    size_t bytes = 0;
    bool busy = false;
};

// One frame of a launch whose results the emit kernel writes to host memory.
struct SrvEmitItem {
    int slot;
    int per;                      // match block stride (entries per level); 0: the frame has no pair
    const int32_t* matches;       // the pair's match blocks
    const uint32_t* match_count;  // the pair's per-level match counts
    uint32_t* out;                // device address of the slot's mapped host result area
};

// Words of a result area before the feature records: kept[L], raw[L],
// matches[L] (clamped to the block stride), padded to 16 bytes.
__host__ __device__ inline int res_header_words(int L) { return (3 * L + 3) / 4 * 4; }

// Result area of one frame (pinned host memory, written by the device):
// header, then every kept feature (48 B) level by level, then every match
// (16 B) level by level -- what uslam_server_result hands out, so the
// results reach host memory with the launch and a result call reads no
// device memory.
__global__ void __launch_bounds__(256) k_server_emit(const FrameDev* __restrict__ frames,
                                                      const SrvEmitItem* __restrict__ items, int L) {
    __shared__ uint32_t s_cnt[2][USLAM_MAX_LEVELS];
    __shared__ uint32_t s_off[2][USLAM_MAX_LEVELS + 1];
    const SrvEmitItem it = items[blockIdx.x];
    const FrameDev& F = frames[it.slot];
    const int hw = res_header_words(L);
    if (threadIdx.x == 0) {
        uint32_t fo = 0, mo = 0;
        for (int l = 0; l < L; ++l) {
            const uint32_t k = F.kept[l];
            const uint32_t m = it.per > 0 ? min(it.match_count[l], (uint32_t)it.per) : 0u;
            s_cnt[0][l] = k;
            s_cnt[1][l] = m;
            s_off[0][l] = fo;
            s_off[1][l] = mo;
            fo += k;
            mo += m;
            it.out[l] = k;
            it.out[L + l] = F.raw[l];
            it.out[2 * L + l] = m;
        }
        s_off[0][L] = fo;
        s_off[1][L] = mo;
        for (int q = 3 * L; q < hw; ++q) it.out[q] = 0u;
    }
    __syncthreads();
    uint4* fdst = reinterpret_cast<uint4*>(it.out + hw);
    uint4* mdst = fdst + 3u * s_off[0][L];
    for (int l = 0; l < L; ++l) {
        const uint4* src = reinterpret_cast<const uint4*>(F.feats[l]);
        uint4* dst = fdst + 3u * s_off[0][l];
        for (uint32_t i = threadIdx.x; i < 3u * s_cnt[0][l]; i += blockDim.x) dst[i] = src[i];
        if (it.per > 0) {
            const uint4* msrc = reinterpret_cast<const uint4*>(it.matches) + (size_t)l * it.per;
            uint4* md = mdst + s_off[1][l];
            for (uint32_t i = threadIdx.x; i < s_cnt[1][l]; i += blockDim.x) md[i] = msrc[i];
        }
    }
}

}  // namespace

struct uslam_server {
    uslam_ctx* ctx = nullptr;
    int levels = 0;
    int max_batch = 0;
    std::vector<SrvClass> classes;
    std::vector<SrvSlot> slots;
    std::vector<FrameDev> frames;
    FrameDev* d_frames = nullptr;
    char* arena = nullptr;
    uint32_t* d_err = nullptr;
    uint32_t* h_err = nullptr;  // pinned: the error word as of the end of each table buffer's last launch
    int max_w = 0;
    cudaStream_t cs[2] = {nullptr, nullptr};
    LaunchBuf bufs[2];
    std::vector<SrvStream> streams;
    std::unordered_map<uint64_t, SrvReq> reqs;
    std::deque<uint64_t> pending;
    std::deque<SrvLaunch> inflight;
    uint64_t next_ticket = 1;
    int next_launch = 0;
    uint64_t n_launches = 0, n_frames = 0;
    int max_batch_seen = 0;
    std::string fatal;  // first dispatcher failure
    uslam_status fatal_status = USLAM_OK;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::thread worker;
};

namespace {

size_t tables_bytes(int max_batch, int max_tiles_per_frame, int max_bands_per_frame, int max_desc_per_frame,
                    int levels) {
    const size_t t = round_up(sizeof(TileItem) * static_cast<size_t>(max_batch) * max_tiles_per_frame, 256);
    const size_t f = round_up(sizeof(SegDev) * static_cast<size_t>(max_batch) * levels, 256);
    const size_t m = round_up(sizeof(MatchSegDev) * static_cast<size_t>(max_batch) * levels, 256);
    const size_t u = round_up(sizeof(SegDev) * static_cast<size_t>(max_batch) * levels, 256);
    const size_t p = round_up(sizeof(PairDev) * static_cast<size_t>(max_batch), 256);
    const size_t b = round_up(sizeof(BandItem) * static_cast<size_t>(max_batch) * max_bands_per_frame, 256);
    const size_t x = round_up(sizeof(SrvEmitItem) * static_cast<size_t>(max_batch), 256);
    const size_t d = round_up(sizeof(BandItem) * static_cast<size_t>(max_batch) * max_desc_per_frame, 256);
    return t + f + m + u + p + b + x + d;
}

void free_server(uslam_server* s) {
    if (!s) return;
    for (auto& b : s->bufs) {
        if (b.h) cudaFreeHost(b.h);
        if (b.d) cudaFree(b.d);
    }
    for (auto& L : s->inflight)
        if (L.done) cudaEventDestroy(L.done);
    for (auto& sl : s->slots) {
        if (sl.h_in) cudaFreeHost(sl.h_in);
        if (sl.h_res) cudaFreeHost(sl.h_res);
    }
    for (auto& c : s->cs)
        if (c) cudaStreamDestroy(c);
    if (s->arena) cudaFree(s->arena);
    if (s->h_err) cudaFreeHost(s->h_err);
    delete s;
}

// A slot is free when no request owns it, no stream holds it as keyframe,
// no queued/in-flight request matches against it and no launch writes it.
bool slot_free(const SrvSlot& sl) { return !sl.in_use && !sl.keyframe && sl.refs == 0 && sl.producer_launch < 0; }

// Build and enqueue one launch over `tickets` (called with the lock held).
cudaError_t launch_batch(uslam_server* s, const std::vector<uint64_t>& tickets, int bufi, SrvLaunch* L) {
    uslam_ctx* c = s->ctx;
    LaunchBuf& B = s->bufs[bufi];
    cudaStream_t st = s->cs[bufi];
    const int lv = s->levels;
    ShapedTiles shaped;
    std::vector<SegDev> fsegs, usegs;
    std::vector<MatchSegDev> msegs;
    std::vector<PairDev> pairs;
    std::vector<BandItem> bands, desc;
    std::vector<SrvEmitItem> emits;
    cudaError_t e = cudaSuccess;
    for (uint64_t tk : tickets) {
        SrvReq& r = s->reqs[tk];
        SrvSlot& sl = s->slots[r.slot];
        const SrvClass& C = s->classes[sl.cls];
        SrvEmitItem em{};
        em.slot = r.slot;
        em.out = sl.d_res;
        if (r.ref >= 0) {
            em.per = std::max(s->frames[r.ref].cap, 1);
            em.matches = sl.matches;
            em.match_count = sl.match_count;
        }
        emits.push_back(em);
        for (TileItem t : C.tiles) {
            t.frame = static_cast<uint16_t>(r.slot);
            shaped.by_shape[C.shape].push_back(t);
        }
        for (int l = 0; l < lv; ++l) fsegs.push_back(SegDev{r.slot, l});
        for (BandItem bi : C.bands) {
            bi.frame = static_cast<uint16_t>(r.slot);
            bands.push_back(bi);
        }
        for (BandItem bi : C.desc) {
            bi.frame = static_cast<uint16_t>(r.slot);
            desc.push_back(bi);
        }
        const FrameDev& F = s->frames[r.slot];
        e = cudaMemcpyAsync(const_cast<uint8_t*>(F.img), sl.h_in, static_cast<size_t>(F.H0) * F.img_pitch,
                            cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return e;
        if (r.ref >= 0) {
            // the keyframe may be produced by a launch still in flight on the other stream
            const int pl = s->slots[r.ref].producer_launch;
            if (pl >= 0 && pl != L->id) {
                for (auto& other : s->inflight)
                    if (other.id == pl) {
                        e = cudaStreamWaitEvent(st, other.done, 0);
                        if (e != cudaSuccess) return e;
                    }
            }
            PairDev P{};
            P.prev = r.ref;
            P.curr = r.slot;
            P.a2b = sl.a2b;
            P.bacc = sl.bacc;
            P.matches = sl.matches;
            P.match_count = sl.match_count;
            P.max_matches_per_level = std::max(s->frames[r.ref].cap, 1);
            P.max_dx = 0.1f * static_cast<float>(static_cast<uint32_t>(F.W0));
            P.max_dy = 0.1f * static_cast<float>(static_cast<uint32_t>(F.H0));
            const int pi = static_cast<int>(pairs.size());
            pairs.push_back(P);
            for (int l = 0; l < lv; ++l) {
                msegs.push_back(MatchSegDev{pi, 1, l});  // both directions from the keyframe's queries
                usegs.push_back(SegDev{pi, l});
            }
        }
    }
    shaped.finish();
    const std::vector<TileItem>& tiles = shaped.flat;
    // table image: tiles | fsegs | msegs | usegs | pairs | bands | emits | describe items
    const size_t t_b = round_up(tiles.size() * sizeof(TileItem), 256);
    const size_t f_b = round_up(fsegs.size() * sizeof(SegDev), 256);
    const size_t m_b = round_up(msegs.size() * sizeof(MatchSegDev), 256);
    const size_t u_b = round_up(usegs.size() * sizeof(SegDev), 256);
    const size_t p_b = round_up(pairs.size() * sizeof(PairDev), 256);
    const size_t b_b = round_up(bands.size() * sizeof(BandItem), 256);
    const size_t x_b = round_up(emits.size() * sizeof(SrvEmitItem), 256);
    const size_t d_b = round_up(desc.size() * sizeof(BandItem), 256);
    if (t_b + f_b + m_b + u_b + p_b + b_b + x_b + d_b > B.bytes) return cudaErrorInvalidValue;
    char* h = B.h;
    std::memcpy(h, tiles.data(), tiles.size() * sizeof(TileItem));
    std::memcpy(h + t_b, fsegs.data(), fsegs.size() * sizeof(SegDev));
    std::memcpy(h + t_b + f_b, msegs.data(), msegs.size() * sizeof(MatchSegDev));
    std::memcpy(h + t_b + f_b + m_b, usegs.data(), usegs.size() * sizeof(SegDev));
    std::memcpy(h + t_b + f_b + m_b + u_b, pairs.data(), pairs.size() * sizeof(PairDev));
    std::memcpy(h + t_b + f_b + m_b + u_b + p_b, bands.data(), bands.size() * sizeof(BandItem));
    std::memcpy(h + t_b + f_b + m_b + u_b + p_b + b_b, emits.data(), emits.size() * sizeof(SrvEmitItem));
    std::memcpy(h + t_b + f_b + m_b + u_b + p_b + b_b + x_b, desc.data(), desc.size() * sizeof(BandItem));
    const size_t total = t_b + f_b + m_b + u_b + p_b + b_b + x_b + d_b;
    e = cudaMemcpyAsync(B.d, h, total, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    const auto* d_tiles = reinterpret_cast<const TileItem*>(B.d);
    const auto* d_fsegs = reinterpret_cast<const SegDev*>(B.d + t_b);
    const auto* d_msegs = B.d + t_b + f_b;
    const auto* d_usegs = reinterpret_cast<const SegDev*>(B.d + t_b + f_b + m_b);
    const auto* d_pairs = reinterpret_cast<const PairDev*>(B.d + t_b + f_b + m_b + u_b);
    const auto* d_bands = reinterpret_cast<const BandItem*>(B.d + t_b + f_b + m_b + u_b + p_b);
    const auto* d_emits = reinterpret_cast<const SrvEmitItem*>(B.d + t_b + f_b + m_b + u_b + p_b + b_b);
    const auto* d_desc = reinterpret_cast<const BandItem*>(B.d + t_b + f_b + m_b + u_b + p_b + b_b + x_b);
    const int grid = c->num_sms * 4;
    const int nf = static_cast<int>(fsegs.size());
    if ((e = launch_detect_shaped(s->d_frames, d_tiles, shaped.begin, c->detector, s->d_err, st)) != cudaSuccess) return e;
    if ((e = launch_blur_border(s->d_frames, d_fsegs, nf, grid, st)) != cudaSuccess) return e;
    if ((e = launch_compact_banded(s->d_frames, d_bands, static_cast<int>(bands.size()), d_fsegs, nf, s->max_w,
                                   st)) != cudaSuccess)
        return e;
    e = c->describe_form == 1 && static_cast<int>(emits.size()) >= kTiledDescribeFrames &&
                describe_tiled_smem(c->margin) > 0
            ? launch_describe_tiled(s->d_frames, d_desc, static_cast<int>(desc.size()), c->d_pattern, false, false,
                                    c->margin, s->d_err, st)
            : launch_describe(s->d_frames, d_fsegs, nf, c->d_pattern, grid, false, false, st);
    if (e != cudaSuccess) return e;
    if (!pairs.empty()) {
        if ((e = launch_bacc_init(s->d_frames, d_pairs, d_usegs, static_cast<int>(usegs.size()), st)) != cudaSuccess)
            return e;
        if ((e = launch_match(s->d_frames, d_pairs, d_msegs, static_cast<int>(msegs.size()), c->num_sms, st)) !=
            cudaSuccess)
            return e;
        if ((e = launch_mutual(s->d_frames, d_pairs, d_usegs, static_cast<int>(usegs.size()), s->d_err, st)) !=
            cudaSuccess)
            return e;
    }
    // every frame's features and matches to its slot's host result area
    k_server_emit<<<static_cast<int>(emits.size()), 256, 0, st>>>(s->d_frames, d_emits, lv);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // the error word (kernel bounds checks, tile-load wait limits) travels
    // with the launch and is read when the launch completes
    if ((e = cudaMemcpyAsync(&s->h_err[bufi], s->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    return cudaEventRecord(L->done, st);
}

void dispatcher(uslam_server* s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop) {
        // completions
        bool progressed = false;
        while (!s->inflight.empty()) {
            SrvLaunch& L = s->inflight.front();
            const cudaError_t q = cudaEventQuery(L.done);
            if (q == cudaErrorNotReady) break;
            if (q != cudaSuccess && s->fatal.empty()) {
                s->fatal = std::string("launch failed: ") + cudaGetErrorString(q);
                s->fatal_status = USLAM_CUDA_ERROR;
            }
            if (q == cudaSuccess && s->h_err[L.buf] != 0u && s->fatal.empty()) {
                s->fatal = "kernel check tripped (error word " + std::to_string(s->h_err[L.buf]) + ")";
                s->fatal_status = USLAM_KERNEL_CHECK;
            }
            const auto now = Clock::now();
            const bool failed = q != cudaSuccess || s->h_err[L.buf] != 0u;
            for (uint64_t tk : L.tickets) {
                SrvReq& r = s->reqs[tk];
                r.done = true;
                r.failed = failed;
                r.t_done = now;
                if (s->slots[r.slot].producer_launch == L.id) s->slots[r.slot].producer_launch = -1;
                if (r.ref >= 0) --s->slots[r.ref].refs;
            }
            s->bufs[L.buf].busy = false;
            cudaEventDestroy(L.done);
            s->inflight.pop_front();
            progressed = true;
        }
        if (progressed) s->cv_done.notify_all();
        if (!s->fatal.empty() && !s->pending.empty()) {
            // after a failure nothing more is launched: what is queued
            // finishes now, and its waiters see the failure
            const auto now = Clock::now();
            while (!s->pending.empty()) {
                const auto it = s->reqs.find(s->pending.front());
                s->pending.pop_front();
                if (it == s->reqs.end()) continue;
                it->second.done = true;
                it->second.failed = true;
                it->second.t_done = now;
                if (it->second.ref >= 0) --s->slots[it->second.ref].refs;
            }
            s->cv_done.notify_all();
        }
        // launch whatever is queued on a free table buffer
        int bufi = !s->bufs[0].busy ? 0 : (!s->bufs[1].busy ? 1 : -1);
        if (!s->pending.empty() && bufi >= 0 && s->fatal.empty()) {
            std::vector<uint64_t> batch;
            while (!s->pending.empty() && static_cast<int>(batch.size()) < s->max_batch) {
                batch.push_back(s->pending.front());
                s->pending.pop_front();
            }
            SrvLaunch L;
            L.id = s->next_launch++;
            L.buf = bufi;
            L.tickets = batch;
            cudaError_t e = cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming);
            for (uint64_t tk : batch) s->slots[s->reqs[tk].slot].producer_launch = L.id;
            if (e == cudaSuccess) e = launch_batch(s, batch, bufi, &L);
            if (e != cudaSuccess) {
                if (s->fatal.empty()) {
                    s->fatal = std::string("launch: ") + cudaGetErrorString(e);
                    s->fatal_status = USLAM_CUDA_ERROR;
                }
                if (L.done) cudaEventDestroy(L.done);
                const auto now = Clock::now();
                for (uint64_t tk : batch) {
                    SrvReq& r = s->reqs[tk];
                    r.done = true;
                    r.failed = true;
                    r.t_done = now;
                    s->slots[r.slot].producer_launch = -1;
                    if (r.ref >= 0) --s->slots[r.ref].refs;
                }
                s->cv_done.notify_all();
                continue;
            }
            s->bufs[bufi].busy = true;
            ++s->n_launches;
            s->n_frames += batch.size();
            s->max_batch_seen = std::max(s->max_batch_seen, static_cast<int>(batch.size()));
            s->inflight.push_back(std::move(L));
            continue;
        }
        // nothing to launch: wait for a submission, or poll in-flight work
        if (s->inflight.empty())
            s->cv_work.wait(lk, [s] { return s->stop || !s->pending.empty(); });
        else {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        }
    }
}

}  // namespace

extern "C" {

uslam_status uslam_server_create(uslam_ctx* ctx, const uslam_server_params* p, uslam_server** out) {
    if (!ctx || !p || !out || p->n_sizes < 1 || !p->widths || !p->heights || p->max_batch < 1 || p->max_batch > 4096)
        return set_err(ctx ? &ctx->err : nullptr, USLAM_INVALID_ARG, "server_create: bad arguments");
    if (ctx->matcher != 0)
        return set_err(&ctx->err, USLAM_INVALID_ARG, "server_create: the served form runs the windowed matcher only");
    // one launch holds max_batch frames: its (frame, level) and (pair, level)
    // segment tables must fit the persistent kernels' shared prefix tables
    if (static_cast<long long>(p->max_batch) * ctx->levels > USLAM_MAX_MATCH_SEGS)
        return set_err(&ctx->err, USLAM_INVALID_ARG, "server_create: max_batch x levels exceeds 2048");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaSetDevice");
    auto* s = new uslam_server();
    s->ctx = ctx;
    s->levels = ctx->levels;
    s->max_batch = p->max_batch;
    const int L = ctx->levels;
    // slot bytes per class, then slots per class from an equal share of the budget
    struct SlotLayout {
        size_t bytes, in, counts, lvl[USLAM_MAX_LEVELS], blur[USLAM_MAX_LEVELS], kpmap[USLAM_MAX_LEVELS],
            feats[USLAM_MAX_LEVELS], xorder[USLAM_MAX_LEVELS], colstart[USLAM_MAX_LEVELS], qorder[USLAM_MAX_LEVELS], bands[USLAM_MAX_LEVELS], a2b, bacc, matches, mcount,
            tmaps;
    };
    std::vector<SlotLayout> lay(p->n_sizes);
    std::vector<FrameDev> proto(p->n_sizes);
    int max_tiles = 1, max_bands = 1, max_desc = 1;
    for (int k = 0; k < p->n_sizes; ++k) {
        const int W0 = p->widths[k], H0 = p->heights[k];
        if (W0 < 1 || H0 < 1 || W0 > ctx->max_w || H0 > ctx->max_h) {
            free_server(s);
            return set_err(&ctx->err, USLAM_INVALID_ARG, "server_create: size class outside the context's limits");
        }
        FrameDev& F = proto[k];
        std::memset(&F, 0, sizeof F);
        F.W0 = W0;
        F.H0 = H0;
        F.levels = L;
        F.margin = ctx->margin;
        F.cell_cap = ctx->cell_cap;
        F.frame_cap = ctx->frame_cap;
        F.detect_first_wait = F.match_first_wait = -1;
        F.img_pitch = static_cast<int>(round_up(static_cast<size_t>(W0), 16));
        level_dims(W0, H0, L, F.w, F.h);
        for (int l = 0; l < L; ++l)
            if (F.w[l] < 1 || F.h[l] < 1) {
                free_server(s);
                return set_err(&ctx->err, USLAM_INVALID_ARG, "server_create: empty pyramid level");
            }
        F.cap = ctx->cap_override > 0 ? ctx->cap_override : static_cast<int>(static_cast<long long>(W0) * H0 / 250);
        const size_t capa = static_cast<size_t>(std::max(F.cap, 1));
        SlotLayout& Y = lay[k];
        size_t cur = 0;
        auto take = [&cur](size_t n) {
            const size_t o = round_up(cur, 256);
            cur = o + n;
            return o;
        };
        Y.in = take(static_cast<size_t>(H0) * F.img_pitch);
        Y.counts = take(2 * sizeof(uint32_t) * L);
        SrvClass C;
        C.W0 = W0;
        C.H0 = H0;
        for (int l = 0; l < L; ++l) {
            F.kp_pitch[l] = static_cast<int>(round_up(static_cast<size_t>(F.w[l]), 16));
            F.bl_pitch[l] = lvl_pitch_of(F.w[l] + ctx->margin + 1);  // 16-byte rows (TMA)
            F.lvl_pitch[l] = lvl_pitch_of(F.w[l]);
            Y.feats[l] = take(capa * 48);
            Y.lvl[l] = take(static_cast<size_t>(F.h[l]) * F.lvl_pitch[l] * 4);
            Y.blur[l] = take(static_cast<size_t>(F.h[l] + ctx->margin + 1) * F.bl_pitch[l] * 4);
            Y.kpmap[l] = take(static_cast<size_t>(F.h[l]) * F.kp_pitch[l]);
            Y.xorder[l] = take(USLAM_MATCH_BANDS * capa * 4);
            Y.colstart[l] = take((USLAM_MATCH_BANDS * (static_cast<size_t>(F.w[l]) + 1) + USLAM_MATCH_BANDS + 1) * 4);
            Y.qorder[l] = take(capa * 4);
            Y.bands[l] = take(static_cast<size_t>((F.h[l] + 31) / 32) * 8);
        }
        C.shape = ctx->shape_for(W0, H0);
        append_tiles(&C.tiles, 0, F, C.shape);
        for (int l = 0; l < L; ++l)
            for (int q = 0; q < (F.h[l] + 31) / 32; ++q) {
                BandItem bi{};
                bi.level = static_cast<uint8_t>(l);
                bi.band = static_cast<uint16_t>(q);
                C.bands.push_back(bi);
                for (int ch = 0; ch < (F.w[l] + KDT_CW - 1) / KDT_CW; ++ch) {
                    bi.pad2 = static_cast<uint16_t>(ch);
                    C.desc.push_back(bi);
                }
            }
        Y.a2b = take(static_cast<size_t>(L) * capa * 4);
        Y.bacc = take(static_cast<size_t>(L) * capa * 16);
        Y.matches = take(static_cast<size_t>(L) * capa * 16);
        Y.mcount = take(sizeof(uint32_t) * L);
        Y.tmaps = take(static_cast<size_t>(L) * USLAM_TMAPS_PER_LEVEL * USLAM_TMAP_BYTES);
        Y.bytes = round_up(cur, 256);
        C.tiles_per_frame = static_cast<int>(C.tiles.size());
        max_tiles = std::max(max_tiles, C.tiles_per_frame);
        max_bands = std::max(max_bands, static_cast<int>(C.bands.size()));
        max_desc = std::max(max_desc, static_cast<int>(C.desc.size()));
        s->max_w = std::max(s->max_w, F.w[0]);
        s->classes.push_back(std::move(C));
    }
    const size_t share = p->hbm_budget_bytes / static_cast<size_t>(p->n_sizes);
    size_t arena = 256;
    int nslots = 0;
    for (int k = 0; k < p->n_sizes; ++k) {
        const int n = static_cast<int>(std::min<size_t>(share / lay[k].bytes, 65535 / p->n_sizes));
        if (n < 2) {
            free_server(s);
            return set_err(&ctx->err, USLAM_CAPACITY, "server_create: the HBM budget holds fewer than 2 slots of a size class");
        }
        s->classes[k].first_slot = nslots;
        s->classes[k].n_slots = n;
        nslots += n;
        arena += lay[k].bytes * n;
    }
    e = cudaMalloc(&s->arena, arena);
    if (e != cudaSuccess) {
        cudaGetLastError();
        free_server(s);
        return set_err(&ctx->err, USLAM_OOM, "server_create: arena allocation refused");
    }
    e = cudaMemset(s->arena, 0, arena);
    s->d_err = reinterpret_cast<uint32_t*>(s->arena);
    s->slots.resize(nslots);
    s->frames.resize(nslots);
    size_t off = 256;
    for (int k = 0; k < p->n_sizes && e == cudaSuccess; ++k) {
        std::vector<uint32_t*> masks;
        uslam_status ms = ctx->masks_for(proto[k].W0, proto[k].H0, proto[k].w, proto[k].h, &masks);
        if (ms != USLAM_OK) {
            free_server(s);
            return ms;
        }
        for (int i = 0; i < s->classes[k].n_slots; ++i, off += lay[k].bytes) {
            const int g = s->classes[k].first_slot + i;
            char* base = s->arena + off;
            const SlotLayout& Y = lay[k];
            FrameDev F = proto[k];
            F.img = reinterpret_cast<const uint8_t*>(base + Y.in);
            F.kept = reinterpret_cast<uint32_t*>(base + Y.counts);
            F.raw = F.kept + L;
            for (int l = 0; l < L; ++l) {
                F.lvl[l] = reinterpret_cast<float*>(base + Y.lvl[l]);
                F.blur[l] = reinterpret_cast<float*>(base + Y.blur[l]);
                F.kpmap[l] = reinterpret_cast<uint8_t*>(base + Y.kpmap[l]);
                F.feats[l] = reinterpret_cast<uint32_t*>(base + Y.feats[l]);
                F.xorder[l] = reinterpret_cast<uint32_t*>(base + Y.xorder[l]);
                F.colstart[l] = reinterpret_cast<uint32_t*>(base + Y.colstart[l]);
                F.qorder[l] = reinterpret_cast<uint32_t*>(base + Y.qorder[l]);
                F.bands[l] = reinterpret_cast<uint32_t*>(base + Y.bands[l]);
                F.mask[l] = masks[l];
            }
            F.tmaps = base + Y.tmaps;
            std::vector<char> maps(static_cast<size_t>(L) * USLAM_TMAPS_PER_LEVEL * USLAM_TMAP_BYTES);
            const uslam_status ts = encode_tile_maps(F, ctx->detector, maps.data(), &ctx->err);
            if (ts != USLAM_OK) {
                free_server(s);
                return ts;
            }
            e = cudaMemcpy(base + Y.tmaps, maps.data(), maps.size(), cudaMemcpyHostToDevice);
            s->frames[g] = F;
            SrvSlot& sl = s->slots[g];
            sl.cls = k;
            sl.a2b = reinterpret_cast<int32_t*>(base + Y.a2b);
            sl.bacc = reinterpret_cast<uint4*>(base + Y.bacc);
            sl.matches = reinterpret_cast<int32_t*>(base + Y.matches);
            sl.match_count = reinterpret_cast<uint32_t*>(base + Y.mcount);
            if (e == cudaSuccess) e = cudaHostAlloc(&sl.h_in, static_cast<size_t>(F.H0) * F.img_pitch, cudaHostAllocDefault);
            // results: header, every feature the slot can keep, every match of its
            // pair (a keyframe of the same size class has the same cap)
            const size_t capr = static_cast<size_t>(std::max(F.cap, 1)) * L;
            const size_t res_bytes = 4 * static_cast<size_t>(res_header_words(L)) + 48 * capr + 16 * capr;
            if (e == cudaSuccess)
                e = cudaHostAlloc(&sl.h_res, res_bytes, cudaHostAllocMapped | cudaHostAllocPortable);
            if (e == cudaSuccess) e = cudaHostGetDevicePointer(&sl.d_res, sl.h_res, 0);
        }
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->d_frames, sizeof(FrameDev) * nslots);
    if (e == cudaSuccess)
        e = cudaMemcpy(s->d_frames, s->frames.data(), sizeof(FrameDev) * nslots, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_err, 2 * sizeof(uint32_t), cudaHostAllocDefault);
    if (e == cudaSuccess) s->h_err[0] = s->h_err[1] = 0u;
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        s->bufs[b].bytes = tables_bytes(s->max_batch, max_tiles, max_bands, max_desc, L);
        e = cudaHostAlloc(&s->bufs[b].h, s->bufs[b].bytes, cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaMalloc(&s->bufs[b].d, s->bufs[b].bytes);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cs[b], cudaStreamNonBlocking);
    }
    if (e == cudaSuccess) e = set_compact_smem(s->max_w);
    if (e == cudaSuccess && ctx->describe_form == 1 && describe_tiled_smem(ctx->margin) > 0)
        e = set_describe_tiled_smem(ctx->margin);
    if (e != cudaSuccess) {
        const std::string m = std::string("server_create: ") + cudaGetErrorString(e);
        cudaGetLastError();
        if (s->d_frames) cudaFree(s->d_frames);
        free_server(s);
        return set_err(&ctx->err, e == cudaErrorMemoryAllocation ? USLAM_OOM : USLAM_CUDA_ERROR, m);
    }
    s->worker = std::thread(dispatcher, s);
    *out = s;
    return USLAM_OK;
}

void uslam_server_destroy(uslam_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    for (auto& c : s->cs)
        if (c) cudaStreamSynchronize(c);
    if (s->d_frames) cudaFree(s->d_frames);
    free_server(s);
}

uslam_status uslam_server_open_stream(uslam_server* s, int width, int height, int* stream_id) {
    if (!s || !stream_id) return USLAM_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    for (size_t k = 0; k < s->classes.size(); ++k) {
        if (s->classes[k].W0 == width && s->classes[k].H0 == height) {
            SrvStream st;
            st.cls = static_cast<int>(k);
            s->streams.push_back(st);
            *stream_id = static_cast<int>(s->streams.size()) - 1;
            return USLAM_OK;
        }
    }
    return set_err(&s->ctx->err, USLAM_INVALID_ARG, "open_stream: no size class for that frame size");
}

uslam_status uslam_server_submit(uslam_server* s, int stream, const uint8_t* img, int pitch, int promote_keyframe,
                                 uint64_t* ticket) {
    if (!s || !img || !ticket) return USLAM_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (stream < 0 || stream >= static_cast<int>(s->streams.size()))
        return set_err(&s->ctx->err, USLAM_INVALID_ARG, "submit: unknown stream");
    if (!s->fatal.empty()) return set_err(&s->ctx->err, s->fatal_status, s->fatal);
    const SrvClass& C = s->classes[s->streams[stream].cls];
    if (pitch < C.W0) return set_err(&s->ctx->err, USLAM_INVALID_ARG, "submit: pitch smaller than the frame width");
    int slot = -1;
    for (int i = 0; i < C.n_slots; ++i)
        if (slot_free(s->slots[C.first_slot + i])) {
            slot = C.first_slot + i;
            break;
        }
    if (slot < 0) return set_err(&s->ctx->err, USLAM_CAPACITY, "submit: no free slot of this size (HBM budget)");
    SrvSlot& sl = s->slots[slot];
    const FrameDev& F = s->frames[slot];
    // reserve the slot, copy the frame into its pinned staging without the
    // lock (several submitting threads copy in parallel), then queue it
    sl.in_use = true;
    lk.unlock();
    for (int y = 0; y < F.H0; ++y)
        std::memcpy(sl.h_in + static_cast<size_t>(y) * F.img_pitch, img + static_cast<size_t>(y) * pitch, F.W0);
    lk.lock();
    // taken after the copy: open_stream may have grown the stream table meanwhile
    SrvStream& S = s->streams[stream];
    SrvReq r;
    r.stream = stream;
    r.slot = slot;
    r.ref = S.keyframe;
    r.promote = promote_keyframe != 0 || S.keyframe < 0;
    r.t_submit = Clock::now();
    if (r.ref >= 0) ++s->slots[r.ref].refs;
    if (r.promote) {
        if (S.keyframe >= 0) s->slots[S.keyframe].keyframe = false;
        S.keyframe = slot;
        sl.keyframe = true;
    }
    const uint64_t tk = s->next_ticket++;
    s->reqs.emplace(tk, r);
    s->pending.push_back(tk);
    *ticket = tk;
    lk.unlock();
    s->cv_work.notify_one();
    return USLAM_OK;
}

uslam_status uslam_server_wait(uslam_server* s, uint64_t ticket, int timeout_ms) {
    if (!s) return USLAM_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->reqs.find(ticket) == s->reqs.end()) return set_err(&s->ctx->err, USLAM_INVALID_ARG, "wait: unknown ticket");
    // looked up on every wake-up: another thread may release the ticket meanwhile
    auto ready = [&] {
        const auto i = s->reqs.find(ticket);
        return i == s->reqs.end() || i->second.done;
    };
    if (timeout_ms <= 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return set_err(&s->ctx->err, USLAM_TIMEOUT, "wait: request not finished in time");
    }
    if (s->reqs.find(ticket) == s->reqs.end())
        return set_err(&s->ctx->err, USLAM_INVALID_ARG, "wait: ticket released while waiting");
    if (!s->fatal.empty()) return set_err(&s->ctx->err, s->fatal_status, s->fatal);
    return USLAM_OK;
}

uslam_status uslam_server_result(uslam_server* s, uint64_t ticket, uslam_feature* feats, int max_feats, int* kept,
                                 int* raw, uslam_match* matches, int max_matches, int* n_matches, double* latency_ms) {
    if (!s) return USLAM_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || !it->second.done) return set_err(&s->ctx->err, USLAM_NOT_READY, "result: not finished");
    if (it->second.failed) return set_err(&s->ctx->err, s->fatal_status, "result: request failed: " + s->fatal);
    const SrvReq r = it->second;
    const FrameDev F = s->frames[r.slot];
    const SrvSlot sl = s->slots[r.slot];
    lk.unlock();
    const int L = s->levels;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
    // the launch wrote everything to the slot's host result area before its
    // completion event (k_server_emit): no device access here
    (void)F;
    const uint32_t* res = sl.h_res;
    int total = 0, nm = 0;
    for (int l = 0; l < L; ++l) {
        if (kept) kept[l] = static_cast<int>(res[l]);
        if (raw) raw[l] = static_cast<int>(res[L + l]);
        total += static_cast<int>(res[l]);
        nm += static_cast<int>(res[2 * L + l]);
    }
    const uint32_t* frec = res + res_header_words(L);
    if (feats) {
        if (total > max_feats) return set_err(&s->ctx->err, USLAM_CAPACITY, "result: feature buffer too small");
        std::memcpy(feats, frec, sizeof(uslam_feature) * static_cast<size_t>(total));
    }
    if (n_matches) *n_matches = 0;
    if (r.ref < 0) return USLAM_NOT_READY;  // no keyframe to match against (the stream's first frame)
    if (n_matches) *n_matches = nm;
    if (matches) {
        if (nm > max_matches) return set_err(&s->ctx->err, USLAM_CAPACITY, "result: match buffer too small");
        std::memcpy(matches, frec + 12 * static_cast<size_t>(total), sizeof(uslam_match) * static_cast<size_t>(nm));
    }
    return USLAM_OK;
}

uslam_status uslam_server_release(uslam_server* s, uint64_t ticket) {
    if (!s) return USLAM_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_err(&s->ctx->err, USLAM_INVALID_ARG, "release: unknown ticket");
    if (!it->second.done) return set_err(&s->ctx->err, USLAM_NOT_READY, "release: request still running");
    s->slots[it->second.slot].in_use = false;
    s->reqs.erase(it);
    return USLAM_OK;
}

uslam_status uslam_server_stats(uslam_server* s, uint64_t* launches, uint64_t* frames, int* max_batch_seen,
                                int* slots_total) {
    if (!s) return USLAM_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (launches) *launches = s->n_launches;
    if (frames) *frames = s->n_frames;
    if (max_batch_seen) *max_batch_seen = s->max_batch_seen;
    if (slots_total) *slots_total = static_cast<int>(s->slots.size());
    return USLAM_OK;
}

uslam_status uslam_server_set_first_wait(uslam_server* s, int detect_polls) {
    if (!s) return USLAM_INVALID_ARG;
    if (detect_polls < -1) return set_err(&s->ctx->err, USLAM_INVALID_ARG, "set_first_wait: bad arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->inflight.empty() || !s->pending.empty())
        return set_err(&s->ctx->err, USLAM_NOT_READY, "set_first_wait: requests in flight");
    for (FrameDev& F : s->frames) F.detect_first_wait = detect_polls;
    // the kernels read the slot table at run time
    cudaSetDevice(s->ctx->device);
    const cudaError_t e =
        cudaMemcpy(s->d_frames, s->frames.data(), sizeof(FrameDev) * s->frames.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(&s->ctx->err, USLAM_CUDA_ERROR, "set_first_wait: slot table upload");
    }
    return USLAM_OK;
}

}  // extern "C"
