// runtime.cu — host runtime and C ABI of the GB300 feature front-end.
//
// A context (uslam_ctx) owns the device, the BRIEF table and the per-
// resolution cull coverage masks.  A batch (uslam_batch) is a work table over
// frames and frame pairs with every buffer carved out of one arena:
//   [inputs: LOD0 u8 of every frame][outputs: counts + features of every
//   frame, counts + matches of every pair][scratch: pyramid, blur cache,
//   keypoint maps, band counts, the matcher's band lists, match directions,
//   error word]
// so one H2D copy feeds the whole batch and one D2H copy returns it.  The
// batch's launch sequence (k_detect per tile shape; k_blur_border on a forked
// branch beside k_band_count, k_band_write, k_xsort; k_describe; k_match or
// k_bruteforce; k_mutual or the emit) is captured once into a CUDA graph.
// A frontend (uslam_frontend) is a 2-slot batch driven frame by frame with
// the reference's FeatureSet(0)/(1) rotation.
#include <cuda.h>  // CUtensorMap and its encode enums (types only: the entry point comes through the runtime)
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/uslam.h"
#include "uslam_internal.h"

#include "runtime_internal.h"

namespace {

constexpr int kLanes = 2;  // parts of a split batch graph (3 measured no better)

// Batches of at least this many frames are captured as kLanes parts of their
// frames on as many streams (see enqueue_split).
constexpr int kSplitFrames = 16;

// Launch tables of one program (a subset of the batch's frames and pairs).
struct Program {
    int ntiles = 0, nfsegs = 0, nmsegs = 0, nusegs = 0, npsegs = 0, nbands = 0, ndesc = 0;
    BandItem* bands = nullptr;  // compaction work items: one per 32-row band of every (frame, level)
    BandItem* desc = nullptr;   // describe items: every KDT_CW-column chunk of every band
    int tile_begin[kNumTileShapes + 1] = {0};  // tiles grouped by shape
    TileItem* tiles = nullptr;
    SegDev* fsegs = nullptr;
    MatchSegDev* msegs = nullptr;
    SegDev* usegs = nullptr;
    SegDev* psegs = nullptr;  // one (pair, 0) entry per pair (brute-force matcher)
    void* units = nullptr;    // the windowed tensor-core matcher's unit slots (device scratch)
    size_t units_bytes = 0;
    std::vector<char> host;  // host image of the tables
    cudaGraphExec_t graph = nullptr;
};

}  // namespace

struct uslam_batch {
    uslam_ctx* ctx = nullptr;
    int levels = 0;
    int max_w = 0;
    std::vector<FrameDev> frames;
    std::vector<PairDev> pairs;
    std::vector<size_t> in_off;    // per frame, offset of the input in the inputs region
    std::vector<size_t> feat_off;  // per frame, offset of its outputs in the outputs region
    std::vector<size_t> pair_off;  // per pair, offset of its outputs in the outputs region
    char* arena = nullptr;
    size_t in_bytes = 0, out_bytes = 0, arena_bytes = 0;
    char* h_in = nullptr;   // pinned
    char* h_out = nullptr;  // pinned
    FrameDev* d_frames = nullptr;
    PairDev* d_pairs = nullptr;
    uint32_t* d_err = nullptr;
    char* d_tables = nullptr;
    // k_match's claim blocks, one per lane (its counters and claim order),
    // and each lane's group cost buckets
    char* d_claim = nullptr;
    size_t claim_stride = 0, claim_words = 0;
    cudaStream_t stream = nullptr;      // stream in use (own or caller's)
    cudaStream_t own_stream = nullptr;  // created with the batch
    cudaStream_t aux_stream = nullptr;  // k_blur_border's branch beside the compaction
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // graph of a batch of >= kSplitFrames frames: kLanes parts of the frames on
    // as many lanes (streams), so that each part's kernels fill the others' tails
    int nparts = 0;
    Program part[kLanes];
    cudaStream_t lane_st[kLanes] = {}, lane_aux[kLanes] = {};  // lane 0 uses the batch's own streams
    cudaEvent_t lane_fork[kLanes] = {}, lane_join[kLanes] = {}, lane_desc[kLanes] = {}, lane_end[kLanes] = {};
    cudaEvent_t ev_start = nullptr;
    Program full;
    // the windowed matcher on the tensor cores (k_describe<WIN> / k_win_plan /
    // k_win_mma; else k_match): matcher 0 with list positions within 16 bits
    bool win_tc = false;
    int win_umax = 0;  // unit slots per (pair, direction, level)
    std::vector<Program> frame_prog;  // per frame: detect+describe only
    std::vector<Program> pair_prog;   // per pair: match only
    ErrText* err() { return &ctx->err; }
};

namespace {

uslam_status build_program(uslam_batch* b, const std::vector<int>& fr, const std::vector<int>& pr, Program* P) {
    ShapedTiles st;
    std::vector<SegDev> fsegs, usegs, psegs;
    std::vector<MatchSegDev> msegs;
    std::vector<BandItem> bands, desc;
    for (int f : fr) {
        const FrameDev& F = b->frames[f];
        append_tiles(&st.by_shape[b->ctx->shape_for(F.W0, F.H0)], f, F, b->ctx->shape_for(F.W0, F.H0));
        for (int l = 0; l < F.levels; ++l) {
            fsegs.push_back(SegDev{f, l});
            for (int q = 0; q < (F.h[l] + 31) / 32; ++q) {
                BandItem bi{};
                bi.frame = static_cast<uint16_t>(f);
                bi.level = static_cast<uint8_t>(l);
                bi.band = static_cast<uint16_t>(q);
                bands.push_back(bi);
                for (int c = 0; c < (F.w[l] + KDT_CW - 1) / KDT_CW; ++c) {
                    bi.pad2 = static_cast<uint16_t>(c);
                    desc.push_back(bi);
                }
            }
        }
    }
    st.finish();
    const std::vector<TileItem>& tiles = st.flat;
    std::memcpy(P->tile_begin, st.begin, sizeof(P->tile_begin));
    for (int p : pr) {
        psegs.push_back(SegDev{p, 0});
        for (int l = 0; l < b->levels; ++l) {
            usegs.push_back(SegDev{p, l});
            // the tensor-core form takes each direction as its own segment
            if (b->win_tc) {
                msegs.push_back(MatchSegDev{p, 0, l});
                msegs.push_back(MatchSegDev{p, 1, l});
            }
        }
    }
    if (!b->win_tc) {
        // k_match searches both directions from the prev set's queries.  Its
        // warps claim query groups in segment order, so the costliest groups
        // go first and the launch's tail is short: a group's windows cover a
        // fixed share of its frame at about the same feature density, so its
        // cost grows with the frame's area (larger frames first); within one
        // size the groups of the first and last level (two pool levels
        // instead of three) come last (0.594 -> 0.570 ms on the 64-frame step).
        std::vector<int> order;
        for (int l = 1; l + 1 < b->levels; ++l) order.push_back(l);
        order.push_back(0);
        if (b->levels > 1) order.push_back(b->levels - 1);
        std::vector<int> by_area(pr.begin(), pr.end());
        auto area = [&](int p) {
            const FrameDev& F = b->frames[b->pairs[p].curr];
            return static_cast<long long>(F.W0) * F.H0;
        };
        std::stable_sort(by_area.begin(), by_area.end(), [&](int x, int y) { return area(x) > area(y); });
        for (size_t i = 0; i < by_area.size();) {
            size_t j = i;
            while (j < by_area.size() && area(by_area[j]) == area(by_area[i])) ++j;
            for (int l : order)
                for (size_t k = i; k < j; ++k) msegs.push_back(MatchSegDev{by_area[k], 1, l});
            i = j;
        }
    }
    if (static_cast<int>(fsegs.size()) > kMaxSegs || static_cast<int>(msegs.size()) > kMaxSegs)
        return set_err(b->err(), USLAM_CAPACITY, "batch exceeds 4096 (frame, level) or (pair, dir, level) segments");
    if (!b->win_tc && static_cast<int>(msegs.size()) > USLAM_MAX_MATCH_SEGS)
        return set_err(b->err(), USLAM_CAPACITY, "batch exceeds 2048 (pair, level) match segments");
    P->ntiles = static_cast<int>(tiles.size());
    P->nfsegs = static_cast<int>(fsegs.size());
    P->nmsegs = static_cast<int>(msegs.size());
    P->nusegs = static_cast<int>(usegs.size());
    P->npsegs = static_cast<int>(psegs.size());
    P->nbands = static_cast<int>(bands.size());
    P->ndesc = static_cast<int>(desc.size());
    const size_t t_bytes = round_up(tiles.size() * sizeof(TileItem), 256);
    const size_t f_bytes = round_up(fsegs.size() * sizeof(SegDev), 256);
    const size_t m_bytes = round_up(msegs.size() * sizeof(MatchSegDev), 256);
    const size_t u_bytes = round_up(usegs.size() * sizeof(SegDev), 256);
    const size_t p_bytes = round_up(psegs.size() * sizeof(SegDev), 256);
    const size_t b_bytes = round_up(bands.size() * sizeof(BandItem), 256);
    const size_t d_bytes = round_up(desc.size() * sizeof(BandItem), 256);
    P->host.assign(t_bytes + f_bytes + m_bytes + u_bytes + p_bytes + b_bytes + d_bytes, 0);
    std::memcpy(P->host.data(), tiles.data(), tiles.size() * sizeof(TileItem));
    std::memcpy(P->host.data() + t_bytes, fsegs.data(), fsegs.size() * sizeof(SegDev));
    std::memcpy(P->host.data() + t_bytes + f_bytes, msegs.data(), msegs.size() * sizeof(MatchSegDev));
    std::memcpy(P->host.data() + t_bytes + f_bytes + m_bytes, usegs.data(), usegs.size() * sizeof(SegDev));
    std::memcpy(P->host.data() + t_bytes + f_bytes + m_bytes + u_bytes, psegs.data(), psegs.size() * sizeof(SegDev));
    std::memcpy(P->host.data() + t_bytes + f_bytes + m_bytes + u_bytes + p_bytes, bands.data(),
                bands.size() * sizeof(BandItem));
    std::memcpy(P->host.data() + t_bytes + f_bytes + m_bytes + u_bytes + p_bytes + b_bytes, desc.data(),
                desc.size() * sizeof(BandItem));
    // unit slots of the windowed tensor-core matcher: written on the device
    P->units_bytes = b->win_tc ? round_up(msegs.size() * static_cast<size_t>(b->win_umax) * win_unit_bytes(), 256) : 0;
    P->host.resize(P->host.size() + P->units_bytes, 0);
    return USLAM_OK;
}

// A lane of launches: a stream, the stream k_blur_border forks to, their
// fork/join events, and the block k_match claims its query groups from (with
// the group cost buckets its order is built from).
struct Lane {
    cudaStream_t st, aux;
    cudaEvent_t fork, join;
    uint32_t* claim;
    uint8_t* gbucket;
};

uint32_t* lane_claim(uslam_batch* b, int j) {
    return reinterpret_cast<uint32_t*>(b->d_claim + static_cast<size_t>(j) * b->claim_stride);
}
uint8_t* lane_gbucket(uslam_batch* b, int j) {
    return reinterpret_cast<uint8_t*>(b->d_claim + static_cast<size_t>(j) * b->claim_stride) +
           round_up(b->claim_words * sizeof(uint32_t), 256);
}
Lane lane0(uslam_batch* b) {
    return Lane{b->stream, b->aux_stream, b->ev_fork, b->ev_join, lane_claim(b, 0), lane_gbucket(b, 0)};
}

// Describe of a program: the gather form k_describe over (frame, level)
// segments; with describe_form 1, in batches of kTiledDescribeFrames frames
// or more, k_describe_tiled over the describe items (the blur cache staged
// per chunk by TMA) where the pattern's reach fits a TMA box.
bool tiled_describe(const uslam_ctx* c, int n_frames) {
    return c->describe_form == 1 && n_frames >= kTiledDescribeFrames && describe_tiled_smem(c->margin) > 0;
}

cudaError_t describe_stage(uslam_batch* b, const Program& P, cudaStream_t st) {
    uslam_ctx* c = b->ctx;
    if (tiled_describe(c, static_cast<int>(b->frames.size())))
        return launch_describe_tiled(b->d_frames, P.desc, P.ndesc, c->d_pattern, c->matcher == 2, b->win_tc, c->margin,
                                     b->d_err, st);
    return launch_describe(b->d_frames, P.fsegs, P.nfsegs, c->d_pattern, c->num_sms * 4, c->matcher == 2, b->win_tc, st);
}

// The frame stages of a program: pyramid, detect, blur border, compaction, describe.
cudaError_t enqueue_frames(uslam_batch* b, const Program& P, const Lane& ln) {
    uslam_ctx* c = b->ctx;
    cudaError_t e = cudaSuccess;
    if (P.ntiles <= 0) return e;
    if ((e = launch_pyramid_shaped(b->d_frames, P.tiles, P.tile_begin, ln.st)) != cudaSuccess) return e;
    const int grid = c->num_sms * 4;
    // k_blur_border (the blur cache beyond the level edges) reads only the
    // pyramid and the frame, and writes cells k_detect does not: it runs on a
    // forked stream beside k_detect and the compaction and joins before
    // k_describe, which needs both (in a captured graph this is a fork/join).
    if ((e = cudaEventRecord(ln.fork, ln.st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(ln.aux, ln.fork, 0)) != cudaSuccess) return e;
    if ((e = launch_blur_border(b->d_frames, P.fsegs, P.nfsegs, grid, ln.aux)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ln.join, ln.aux)) != cudaSuccess) return e;
    if ((e = launch_detect_only_shaped(b->d_frames, P.tiles, P.tile_begin, c->detector, b->d_err, ln.st)) !=
        cudaSuccess)
        return e;
    if ((e = launch_compact_banded(b->d_frames, P.bands, P.nbands, P.fsegs, P.nfsegs, b->max_w, ln.st)) !=
        cudaSuccess)
        return e;
    if ((e = cudaStreamWaitEvent(ln.st, ln.join, 0)) != cudaSuccess) return e;
    return describe_stage(b, P, ln.st);
}

// The pair stages of a program: match and the mutual check / emit.
cudaError_t enqueue_pairs(uslam_batch* b, const Program& P, const Lane& ln) {
    uslam_ctx* c = b->ctx;
    cudaError_t e = cudaSuccess;
    if (P.nmsegs <= 0) return e;
    const int grid = c->num_sms * 4;
    if (c->matcher != 0) {
        if (c->matcher == 1)
            e = launch_bruteforce(b->d_frames, b->d_pairs, P.psegs, P.npsegs, c->ratio, grid, ln.st);
        else
            e = launch_bf_mma(b->d_frames, b->d_pairs, P.psegs, P.npsegs, c->ratio, c->num_sms, b->d_err, ln.st);
        if (e != cudaSuccess) return e;
        return launch_emit(b->d_frames, b->d_pairs, P.usegs, P.nusegs, b->d_err, ln.st);
    }
    if (b->win_tc) {
        if ((e = launch_win_match(b->d_frames, b->d_pairs, P.msegs, P.nmsegs, b->win_umax, P.units, c->num_sms,
                                  b->d_err, ln.st)) != cudaSuccess)
            return e;
        return launch_mutual(b->d_frames, b->d_pairs, P.usegs, P.nusegs, b->d_err, ln.st);
    }
    if ((e = launch_bacc_init(b->d_frames, b->d_pairs, P.usegs, P.nusegs, ln.st)) != cudaSuccess) return e;
    if ((e = launch_match_dyn(b->d_frames, b->d_pairs, P.msegs, P.nmsegs, c->num_sms, ln.claim, ln.gbucket,
                              ln.st)) != cudaSuccess)
        return e;
    return launch_mutual_reset(b->d_frames, b->d_pairs, P.usegs, P.nusegs, b->d_err, ln.claim, ln.st);
}

// Enqueue a program's launch sequence on the batch stream.
cudaError_t enqueue_program(uslam_batch* b, const Program& P) {
    const Lane ln = lane0(b);
    cudaError_t e = enqueue_frames(b, P, ln);
    return e == cudaSuccess ? enqueue_pairs(b, P, ln) : e;
}

// The split sequence: lane j runs part j's frames, records that its describe
// is done, then waits for the earlier lanes' describe (its pairs may reach
// into their frames) and runs its pairs; lane 0 joins the others at the end.
cudaError_t enqueue_split(uslam_batch* b) {
    const int K = b->nparts;
    Lane ln[kLanes];
    for (int j = 0; j < K; ++j)
        ln[j] = j == 0 ? lane0(b)
                       : Lane{b->lane_st[j], b->lane_aux[j], b->lane_fork[j], b->lane_join[j], lane_claim(b, j),
                              lane_gbucket(b, j)};
    cudaError_t e = cudaEventRecord(b->ev_start, b->stream);
    for (int j = 1; j < K && e == cudaSuccess; ++j) e = cudaStreamWaitEvent(ln[j].st, b->ev_start, 0);
    for (int j = 0; j < K && e == cudaSuccess; ++j) {
        e = enqueue_frames(b, b->part[j], ln[j]);
        if (e == cudaSuccess) e = cudaEventRecord(b->lane_desc[j], ln[j].st);
    }
    for (int j = 0; j < K && e == cudaSuccess; ++j) {
        for (int i = 0; i < j && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(ln[j].st, b->lane_desc[i], 0);
        if (e == cudaSuccess) e = enqueue_pairs(b, b->part[j], ln[j]);
        if (e == cudaSuccess && j > 0) e = cudaEventRecord(b->lane_end[j], ln[j].st);
    }
    for (int j = 1; j < K && e == cudaSuccess; ++j) e = cudaStreamWaitEvent(b->stream, b->lane_end[j], 0);
    return e;
}

uslam_status capture_graph(uslam_batch* b, Program* P) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "begin capture");
    e = cudaMemsetAsync(b->d_err, 0, sizeof(uint32_t), b->stream);
    cudaError_t e2 = e == cudaSuccess ? (b->nparts > 1 && P == &b->full ? enqueue_split(b) : enqueue_program(b, *P)) : e;
    e = cudaStreamEndCapture(b->stream, &g);
    if (e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return b->ctx->cuda_fail(e2, "capture launches");
    }
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "end capture");
    e = cudaGraphInstantiate(&P->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "graph instantiate");
    return USLAM_OK;
}

void free_batch(uslam_batch* b) {
    if (!b) return;
    auto drop = [](Program& P) {
        if (P.graph) cudaGraphExecDestroy(P.graph);
        P.graph = nullptr;
    };
    drop(b->full);
    for (auto& P : b->frame_prog) drop(P);
    for (auto& P : b->pair_prog) drop(P);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    if (b->aux_stream) cudaStreamDestroy(b->aux_stream);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    for (int j = 0; j < kLanes; ++j) {
        for (cudaStream_t st : {b->lane_st[j], b->lane_aux[j]})
            if (st) cudaStreamDestroy(st);
        for (cudaEvent_t ev : {b->lane_fork[j], b->lane_join[j], b->lane_desc[j], b->lane_end[j]})
            if (ev) cudaEventDestroy(ev);
    }
    if (b->ev_start) cudaEventDestroy(b->ev_start);
    if (b->arena) cudaFree(b->arena);
    if (b->d_tables) cudaFree(b->d_tables);
    if (b->d_claim) cudaFree(b->d_claim);
    if (b->h_in) cudaFreeHost(b->h_in);
    if (b->h_out) cudaFreeHost(b->h_out);
    delete b;
}

// per_frame_form: the batch serves the one-frame forms (the frontend, feature
// sets and their matches), where the windowed matcher takes its distances
// from the tensor cores: for one pair k_match leaves most of the GPU idle and
// its latency is that of its slowest query group (measured: the one-frame
// form ran 4,109 frames/s with k_match, 5,497 with k_win_mma).
uslam_status create_batch(uslam_ctx* ctx, int n_frames, const int* widths, const int* heights, int n_pairs,
                          const int* pair_prev, const int* pair_curr, bool per_item_programs, uslam_batch** out,
                          bool per_frame_form = false) {
    if (!ctx || !out || n_frames <= 0 || !widths || !heights || n_pairs < 0 || (n_pairs > 0 && (!pair_prev || !pair_curr)))
        return set_err(ctx ? &ctx->err : nullptr, USLAM_INVALID_ARG, "batch_create: bad arguments");
    if (n_frames > 65535) return set_err(&ctx->err, USLAM_INVALID_ARG, "batch_create: more than 65535 frames");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaSetDevice");
    auto* b = new uslam_batch();
    b->ctx = ctx;
    b->levels = ctx->levels;
    const int L = ctx->levels;
    b->frames.resize(n_frames);
    b->in_off.resize(n_frames);
    b->feat_off.resize(n_frames);
    // ---- layout pass: offsets relative to region starts
    size_t in_bytes = 0, out_bytes = 0, scratch = 0;
    auto take = [](size_t* cur, size_t n) {
        const size_t o = round_up(*cur, 256);
        *cur = o + n;
        return o;
    };
    struct FrameLayout {
        size_t lvl[USLAM_MAX_LEVELS], blur[USLAM_MAX_LEVELS], kpmap[USLAM_MAX_LEVELS], feats[USLAM_MAX_LEVELS],
            xorder[USLAM_MAX_LEVELS], colstart[USLAM_MAX_LEVELS], qorder[USLAM_MAX_LEVELS], bands[USLAM_MAX_LEVELS], counts,
            tmaps, bf8, bfext, bfpop, bfid, wq8, wc8, wcext, wcy, wcid, winv[USLAM_MAX_LEVELS];
    };
    // the windowed tensor-core matcher (matcher 3, or matcher 0 in the
    // one-frame forms): every list position and candidate row within 16 bits,
    // else k_match
    int max_cap = 1;
    for (int f = 0; f < n_frames; ++f) {
        const long long c = ctx->cap_override > 0 ? ctx->cap_override : static_cast<long long>(widths[f]) * heights[f] / 250;
        max_cap = static_cast<int>(std::max<long long>(max_cap, c));
    }
    b->win_tc = (ctx->win_tc || (ctx->matcher == 0 && per_frame_form)) && max_cap <= kWinMaxCap && ctx->max_h < 65535;
    b->win_umax = b->win_tc ? win_units_per_seg(max_cap) : 0;
    std::vector<FrameLayout> fl(n_frames);
    for (int f = 0; f < n_frames; ++f) {
        const int W0 = widths[f], H0 = heights[f];
        if (W0 <= 0 || H0 <= 0 || W0 > ctx->max_w || H0 > ctx->max_h) {
            free_batch(b);
            return set_err(&ctx->err, USLAM_INVALID_ARG,
                           "batch_create: frame " + std::to_string(f) + " size " + std::to_string(W0) + "x" +
                               std::to_string(H0) + " outside 1.." + std::to_string(ctx->max_w) + "x" +
                               std::to_string(ctx->max_h));
        }
        FrameDev& F = b->frames[f];
        std::memset(&F, 0, sizeof(F));
        F.W0 = W0;
        F.H0 = H0;
        F.levels = L;
        F.margin = ctx->margin;
        F.cell_cap = ctx->cell_cap;
        F.frame_cap = ctx->frame_cap;
        F.detect_first_wait = F.match_first_wait = -1;
        F.img_pitch = static_cast<int>(round_up(static_cast<size_t>(W0), 16));
        level_dims(W0, H0, L, F.w, F.h);
        for (int l = 0; l < L; ++l) {
            if (F.w[l] < 1 || F.h[l] < 1) {
                free_batch(b);
                return set_err(&ctx->err, USLAM_INVALID_ARG,
                               "batch_create: frame " + std::to_string(f) + " has an empty pyramid level " +
                                   std::to_string(l));
            }
        }
        const long long cap_ll = ctx->cap_override > 0 ? ctx->cap_override
                                                       : static_cast<long long>(W0) * H0 / 250;
        F.cap = static_cast<int>(cap_ll);
        const size_t capa = static_cast<size_t>(F.cap > 0 ? F.cap : 1);
        b->in_off[f] = take(&in_bytes, static_cast<size_t>(H0) * F.img_pitch);
        b->feat_off[f] = take(&out_bytes, 2 * sizeof(uint32_t) * L);
        FrameLayout& Ly = fl[f];
        Ly.counts = b->feat_off[f];
        for (int l = 0; l < L; ++l) {
            F.kp_pitch[l] = static_cast<int>(round_up(static_cast<size_t>(F.w[l]), 16));
            Ly.feats[l] = take(&out_bytes, capa * 48);
            F.lvl_pitch[l] = lvl_pitch_of(F.w[l]);
            Ly.lvl[l] = take(&scratch, static_cast<size_t>(F.h[l]) * F.lvl_pitch[l] * 4);
            F.bl_pitch[l] = lvl_pitch_of(F.w[l] + ctx->margin + 1);  // 16-byte rows (TMA)
            Ly.blur[l] = take(&scratch, static_cast<size_t>(F.h[l] + ctx->margin + 1) * F.bl_pitch[l] * 4);
            Ly.kpmap[l] = take(&scratch, static_cast<size_t>(F.h[l]) * F.kp_pitch[l]);
            Ly.xorder[l] = take(&scratch, USLAM_MATCH_BANDS * capa * 4);
            Ly.colstart[l] = take(&scratch, (USLAM_MATCH_BANDS * (static_cast<size_t>(F.w[l]) + 1) + USLAM_MATCH_BANDS + 1) * 4);
            Ly.qorder[l] = take(&scratch, capa * 4);
            Ly.bands[l] = take(&scratch, static_cast<size_t>((F.h[l] + 31) / 32) * 8);
        }
        Ly.tmaps = take(&scratch, static_cast<size_t>(L) * USLAM_TMAPS_PER_LEVEL * USLAM_TMAP_BYTES);
        if (ctx->matcher == 2) {
            const size_t rows = tc_rows(F);
            Ly.bf8 = take(&scratch, rows * 256);
            Ly.bfext = take(&scratch, rows * 32);
            Ly.bfpop = take(&scratch, rows * 4);
            Ly.bfid = take(&scratch, rows * 4);
        }
        if (b->win_tc) {
            // queries: each band from a multiple of 128 rows; lists: room for a
            // last 128-row tile that starts below the list's end
            F.wq_rows = static_cast<int>(round_up(capa, 128) + USLAM_MATCH_BANDS * 128);
            F.wc_rows = static_cast<int>(round_up(capa, 32) + 128);
            const size_t qrows = static_cast<size_t>(L) * F.wq_rows;
            const size_t crows = static_cast<size_t>(L) * USLAM_MATCH_BANDS * F.wc_rows;
            Ly.wq8 = take(&scratch, qrows * 256);
            Ly.wc8 = take(&scratch, crows * 256);
            Ly.wcext = take(&scratch, crows * 32);
            Ly.wcy = take(&scratch, crows * 2);
            Ly.wcid = take(&scratch, crows * 4);
            for (int l = 0; l < L; ++l) Ly.winv[l] = take(&scratch, (1 + USLAM_MATCH_BANDS) * capa * 4);
        }
        b->max_w = std::max(b->max_w, F.w[0]);
    }
    b->pairs.resize(n_pairs);
    b->pair_off.resize(n_pairs);
    std::vector<std::pair<size_t, size_t>> dirs(n_pairs);
    // k_match (matcher 0 without the tensor-core form) searches b -> a into
    // per-feature accumulators instead of b2a
    const bool sym_match = ctx->matcher == 0 && !b->win_tc;
    std::vector<size_t> bacc_off(n_pairs, 0);
    for (int p = 0; p < n_pairs; ++p) {
        const int a = pair_prev[p], c = pair_curr[p];
        if (a < 0 || a >= n_frames || c < 0 || c >= n_frames || a == c) {
            free_batch(b);
            return set_err(&ctx->err, USLAM_INVALID_ARG, "batch_create: pair " + std::to_string(p) + " has bad frame indices");
        }
        if (b->frames[a].W0 != b->frames[c].W0 || b->frames[a].H0 != b->frames[c].H0) {
            free_batch(b);
            return set_err(&ctx->err, USLAM_INVALID_ARG, "batch_create: pair " + std::to_string(p) + " mixes frame sizes");
        }
        PairDev& P = b->pairs[p];
        std::memset(&P, 0, sizeof(P));
        P.prev = a;
        P.curr = c;
        const int capa = std::max(b->frames[a].cap, 1), capc = std::max(b->frames[c].cap, 1);
        P.max_matches_per_level = capa;
        // match_features_cpu.cpp:76-77: 0.1F * frame size, in f32
        P.max_dx = 0.1f * static_cast<float>(static_cast<uint32_t>(b->frames[a].W0));
        P.max_dy = 0.1f * static_cast<float>(static_cast<uint32_t>(b->frames[a].H0));
        b->pair_off[p] = take(&out_bytes, round_up(sizeof(uint32_t) * L, 16) + static_cast<size_t>(L) * capa * 16);
        dirs[p].first = take(&scratch, static_cast<size_t>(L) * capa * 4);
        dirs[p].second = take(&scratch, static_cast<size_t>(L) * capc * 4);
        if (sym_match) bacc_off[p] = take(&scratch, static_cast<size_t>(L) * capc * 16);
        P.bf_splits = 1;
        P.bf_ratio = ctx->ratio;
    }
    // Both brute-force matchers take 256 queries per work unit.  Matcher 1
    // runs about 8 CTAs per SM: split each train set until the launch has
    // that many units.  Matcher 2 runs one CTA per SM: pick the smallest
    // split (<= 8) whose units fill at least 95 % of whole waves over the SMs.
    std::vector<size_t> bf_off(n_pairs, 0);
    if (ctx->matcher == 2 && n_pairs > 1024) {
        free_batch(b);
        return set_err(&ctx->err, USLAM_CAPACITY, "batch_create: the tensor-core matcher takes at most 1024 pairs per batch");
    }
    if (ctx->matcher != 0 && n_pairs > 0) {
        size_t units = 0;
        for (int p = 0; p < n_pairs; ++p)
            units += (static_cast<size_t>(L) * std::max(b->frames[pair_prev[p]].cap, 1) + 255) / 256;
        const size_t sms = static_cast<size_t>(std::max(ctx->num_sms, 1));
        int splits = 1;
        if (ctx->matcher == 1) {
            const size_t target = sms * 8;
            splits = static_cast<int>(std::min<size_t>(16, std::max<size_t>(1, (target + units - 1) / units)));
        } else {
            double best_eff = 0.0;
            for (int sp = 1; sp <= 8; ++sp) {
                const size_t u = units * static_cast<size_t>(sp);
                const double eff = static_cast<double>(u) / static_cast<double>((u + sms - 1) / sms * sms);
                if (eff > best_eff + 1e-9) {
                    best_eff = eff;
                    splits = sp;
                }
                if (eff >= 0.95) break;
            }
        }
        if (splits > 1)
            for (int p = 0; p < n_pairs; ++p) {
                b->pairs[p].bf_splits = splits;
                bf_off[p] = take(&scratch, static_cast<size_t>(splits) * L *
                                               std::max(b->frames[pair_prev[p]].cap, 1) * 16);
            }
    }
    const size_t err_off = take(&scratch, 256);  // error word
    const size_t frames_off = take(&scratch, sizeof(FrameDev) * n_frames);
    const size_t pairs_off = take(&scratch, sizeof(PairDev) * std::max(n_pairs, 1));
    in_bytes = round_up(in_bytes, 256);
    out_bytes = round_up(out_bytes, 256);
    b->in_bytes = in_bytes;
    b->out_bytes = out_bytes;
    b->arena_bytes = in_bytes + out_bytes + round_up(scratch, 256);

    e = cudaMalloc(&b->arena, b->arena_bytes);
    if (e != cudaSuccess) {
        const std::string m = std::string("arena of ") + std::to_string(b->arena_bytes) + " bytes: " + cudaGetErrorString(e);
        free_batch(b);
        cudaGetLastError();
        return set_err(&ctx->err, USLAM_OOM, m);
    }
    e = cudaHostAlloc(&b->h_in, in_bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc(&b->h_out, out_bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        free_batch(b);
        cudaGetLastError();
        return set_err(&ctx->err, USLAM_OOM, "pinned staging allocation refused");
    }
    std::memset(b->h_in, 0, in_bytes);
    std::memset(b->h_out, 0, out_bytes);
    e = cudaMemset(b->arena, 0, b->arena_bytes);
    if (e != cudaSuccess) {
        free_batch(b);
        return ctx->cuda_fail(e, "arena clear");
    }
    e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->aux_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        free_batch(b);
        return ctx->cuda_fail(e, "stream create");
    }
    b->stream = b->own_stream;
    char* in_base = b->arena;
    char* out_base = b->arena + in_bytes;
    char* sc_base = b->arena + in_bytes + out_bytes;
    for (int f = 0; f < n_frames; ++f) {
        FrameDev& F = b->frames[f];
        const FrameLayout& Ly = fl[f];
        F.img = reinterpret_cast<const uint8_t*>(in_base + b->in_off[f]);
        F.kept = reinterpret_cast<uint32_t*>(out_base + Ly.counts);
        F.raw = F.kept + L;
        std::vector<uint32_t*> masks;
        uslam_status s = ctx->masks_for(F.W0, F.H0, F.w, F.h, &masks);
        if (s != USLAM_OK) {
            free_batch(b);
            return s;
        }
        for (int l = 0; l < L; ++l) {
            F.lvl[l] = reinterpret_cast<float*>(sc_base + Ly.lvl[l]);
            F.blur[l] = reinterpret_cast<float*>(sc_base + Ly.blur[l]);
            F.kpmap[l] = reinterpret_cast<uint8_t*>(sc_base + Ly.kpmap[l]);
            F.feats[l] = reinterpret_cast<uint32_t*>(out_base + Ly.feats[l]);
            F.xorder[l] = reinterpret_cast<uint32_t*>(sc_base + Ly.xorder[l]);
            F.colstart[l] = reinterpret_cast<uint32_t*>(sc_base + Ly.colstart[l]);
            F.qorder[l] = reinterpret_cast<uint32_t*>(sc_base + Ly.qorder[l]);
            F.bands[l] = reinterpret_cast<uint32_t*>(sc_base + Ly.bands[l]);
            F.mask[l] = masks[l];
        }
        F.tmaps = sc_base + Ly.tmaps;
        if (ctx->matcher == 2) {
            F.bf8 = reinterpret_cast<uint8_t*>(sc_base + Ly.bf8);
            F.bfext = reinterpret_cast<uint8_t*>(sc_base + Ly.bfext);
            F.bfpop = reinterpret_cast<uint32_t*>(sc_base + Ly.bfpop);
            F.bfid = reinterpret_cast<int32_t*>(sc_base + Ly.bfid);
        }
        if (b->win_tc) {
            F.wq8 = reinterpret_cast<uint8_t*>(sc_base + Ly.wq8);
            F.wc8 = reinterpret_cast<uint8_t*>(sc_base + Ly.wc8);
            F.wcext = reinterpret_cast<uint8_t*>(sc_base + Ly.wcext);
            F.wcy = reinterpret_cast<uint16_t*>(sc_base + Ly.wcy);
            F.wcid = reinterpret_cast<int32_t*>(sc_base + Ly.wcid);
            for (int l = 0; l < L; ++l) F.winv[l] = reinterpret_cast<uint32_t*>(sc_base + Ly.winv[l]);
        }
        std::vector<char> maps(static_cast<size_t>(L) * USLAM_TMAPS_PER_LEVEL * USLAM_TMAP_BYTES);
        s = encode_tile_maps(F, ctx->detector, maps.data(), &ctx->err);
        if (s == USLAM_OK) {
            e = cudaMemcpy(sc_base + Ly.tmaps, maps.data(), maps.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) s = ctx->cuda_fail(e, "tensor map upload");
        }
        if (s != USLAM_OK) {
            free_batch(b);
            return s;
        }
    }
    for (int p = 0; p < n_pairs; ++p) {
        PairDev& P = b->pairs[p];
        P.match_count = reinterpret_cast<uint32_t*>(out_base + b->pair_off[p]);
        P.matches = reinterpret_cast<int32_t*>(out_base + b->pair_off[p] + round_up(sizeof(uint32_t) * L, 16));
        P.a2b = reinterpret_cast<int32_t*>(sc_base + dirs[p].first);
        P.b2a = reinterpret_cast<int32_t*>(sc_base + dirs[p].second);
        P.bacc = sym_match ? reinterpret_cast<uint4*>(sc_base + bacc_off[p]) : nullptr;
        P.bf_part = P.bf_splits > 1 ? reinterpret_cast<uint32_t*>(sc_base + bf_off[p]) : nullptr;
    }
    b->d_err = reinterpret_cast<uint32_t*>(sc_base + err_off);
    b->d_frames = reinterpret_cast<FrameDev*>(sc_base + frames_off);
    b->d_pairs = reinterpret_cast<PairDev*>(sc_base + pairs_off);
    e = cudaMemcpy(b->d_frames, b->frames.data(), sizeof(FrameDev) * n_frames, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_pairs > 0)
        e = cudaMemcpy(b->d_pairs, b->pairs.data(), sizeof(PairDev) * n_pairs, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_batch(b);
        return ctx->cuda_fail(e, "frame table upload");
    }
    e = set_compact_smem(b->max_w);
    if (e == cudaSuccess && tiled_describe(ctx, n_frames)) e = set_describe_tiled_smem(ctx->margin);
    if (e == cudaSuccess && ctx->matcher == 2) e = set_bf_mma_smem();
    if (e == cudaSuccess && b->win_tc) e = set_win_mma_smem();
    if (e != cudaSuccess) {
        free_batch(b);
        return ctx->cuda_fail(e, "shared memory attribute");
    }
    // ---- programs
    std::vector<int> all_f(n_frames), all_p(n_pairs);
    for (int f = 0; f < n_frames; ++f) all_f[f] = f;
    for (int p = 0; p < n_pairs; ++p) all_p[p] = p;
    std::vector<Program*> progs;
    uslam_status s = build_program(b, all_f, all_p, &b->full);
    if (s != USLAM_OK) {
        free_batch(b);
        return s;
    }
    progs.push_back(&b->full);
    // (not with matcher 1: its launches are each sized to fill the GPU, and two
    // of them side by side ran the stress step 15 % slower)
    if (n_frames >= kSplitFrames && !per_item_programs && ctx->matcher != 1) {
        // part j: frames [j n / K, (j + 1) n / K) and the pairs whose later frame lies there
        const int K = kLanes;
        auto part_of = [&](int f) { return static_cast<int>(static_cast<long long>(f) * K / n_frames); };
        std::vector<int> fr[kLanes], pr[kLanes];
        for (int f = 0; f < n_frames; ++f) fr[part_of(f)].push_back(f);
        for (int p = 0; p < n_pairs; ++p) pr[std::max(part_of(pair_prev[p]), part_of(pair_curr[p]))].push_back(p);
        for (int j = 0; j < K; ++j) {
            if ((s = build_program(b, fr[j], pr[j], &b->part[j])) != USLAM_OK) {
                free_batch(b);
                return s;
            }
            progs.push_back(&b->part[j]);
        }
        e = cudaEventCreateWithFlags(&b->ev_start, cudaEventDisableTiming);
        for (int j = 0; j < K && e == cudaSuccess; ++j) {
            if (j > 0) {
                e = cudaStreamCreateWithFlags(&b->lane_st[j], cudaStreamNonBlocking);
                if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->lane_aux[j], cudaStreamNonBlocking);
            }
            for (cudaEvent_t* ev : {&b->lane_fork[j], &b->lane_join[j], &b->lane_desc[j], &b->lane_end[j]})
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        }
        if (e != cudaSuccess) {
            free_batch(b);
            return ctx->cuda_fail(e, "stream create");
        }
        b->nparts = K;
    }
    if (per_item_programs) {
        b->frame_prog.resize(n_frames);
        b->pair_prog.resize(n_pairs);
        for (int f = 0; f < n_frames; ++f) {
            if ((s = build_program(b, {f}, {}, &b->frame_prog[f])) != USLAM_OK) {
                free_batch(b);
                return s;
            }
            progs.push_back(&b->frame_prog[f]);
        }
        for (int p = 0; p < n_pairs; ++p) {
            if ((s = build_program(b, {}, {p}, &b->pair_prog[p])) != USLAM_OK) {
                free_batch(b);
                return s;
            }
            progs.push_back(&b->pair_prog[p]);
        }
    }
    // k_match's claim blocks: per lane the counters and an order of up to
    // max_groups query groups (every program's groups are at most the full
    // program's), zeroed once here and by k_mutual after every launch
    {
        size_t max_groups = 0;
        for (int p = 0; p < n_pairs; ++p)
            max_groups += static_cast<size_t>(L) *
                          (static_cast<size_t>(std::max(b->frames[pair_prev[p]].cap, 1)) / 32 + USLAM_MATCH_BANDS + 1);
        b->claim_words = match_claim_words(max_groups);
        b->claim_stride = round_up(b->claim_words * sizeof(uint32_t), 256) + round_up(std::max<size_t>(max_groups, 1), 256);
        e = cudaMalloc(&b->d_claim, b->claim_stride * kLanes);
        if (e == cudaSuccess) e = cudaMemset(b->d_claim, 0, b->claim_stride * kLanes);
        if (e != cudaSuccess) {
            free_batch(b);
            cudaGetLastError();
            return set_err(&ctx->err, USLAM_OOM, "match claim blocks: allocation refused");
        }
    }
    size_t tbytes = 0;
    for (Program* P : progs) tbytes += P->host.size();
    e = cudaMalloc(&b->d_tables, std::max<size_t>(tbytes, 256));
    if (e != cudaSuccess) {
        free_batch(b);
        cudaGetLastError();
        return set_err(&ctx->err, USLAM_OOM, "work table allocation refused");
    }
    size_t cur = 0;
    for (Program* P : progs) {
        char* base = b->d_tables + cur;
        const size_t t_bytes = round_up(P->ntiles * sizeof(TileItem), 256);
        const size_t f_bytes = round_up(P->nfsegs * sizeof(SegDev), 256);
        const size_t m_bytes = round_up(P->nmsegs * sizeof(MatchSegDev), 256);
        const size_t u_bytes = round_up(P->nusegs * sizeof(SegDev), 256);
        P->psegs = reinterpret_cast<SegDev*>(base + t_bytes + f_bytes + m_bytes + u_bytes);
        const size_t p_bytes = round_up(P->npsegs * sizeof(SegDev), 256);
        P->bands = reinterpret_cast<BandItem*>(base + t_bytes + f_bytes + m_bytes + u_bytes + p_bytes);
        const size_t b_bytes = round_up(P->nbands * sizeof(BandItem), 256);
        P->desc = reinterpret_cast<BandItem*>(base + t_bytes + f_bytes + m_bytes + u_bytes + p_bytes + b_bytes);
        P->units = P->units_bytes ? base + (P->host.size() - P->units_bytes) : nullptr;
        P->tiles = reinterpret_cast<TileItem*>(base);
        P->fsegs = reinterpret_cast<SegDev*>(base + t_bytes);
        P->msegs = reinterpret_cast<MatchSegDev*>(base + t_bytes + f_bytes);
        P->usegs = reinterpret_cast<SegDev*>(base + t_bytes + f_bytes + m_bytes);
        if (!P->host.empty()) {
            e = cudaMemcpy(base, P->host.data(), P->host.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                free_batch(b);
                return ctx->cuda_fail(e, "work table upload");
            }
        }
        cur += P->host.size();
    }
    if ((s = capture_graph(b, &b->full)) != USLAM_OK) {
        free_batch(b);
        return s;
    }
    *out = b;
    return USLAM_OK;
}

uslam_status check_err_word(uslam_batch* b) {
    uint32_t word = 0;
    cudaError_t e = cudaMemcpy(&word, b->d_err, sizeof(word), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "error word readback");
    if (word != 0u) {
        std::string m = "kernel bounds check tripped:";
        if (word & USLAM_ERR_SMEM_RANGE) m += " blur tap outside the staged tile;";
        if (word & USLAM_ERR_MATCH_OVERFLOW) m += " match list overflow;";
        if (word & USLAM_ERR_TMA_TIMEOUT) m += " tile load wait limit reached;";
        return set_err(b->err(), USLAM_KERNEL_CHECK, m);
    }
    return USLAM_OK;
}

uslam_status sync_stream(uslam_batch* b, int timeout_ms) {
    cudaError_t e;
    if (timeout_ms <= 0) {
        e = cudaStreamSynchronize(b->stream);
    } else {
        // host watchdog: poll with a deadline instead of blocking forever
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
        while ((e = cudaStreamQuery(b->stream)) == cudaErrorNotReady) {
            if (std::chrono::steady_clock::now() >= deadline)
                return set_err(b->err(), USLAM_TIMEOUT, "batch did not finish within " + std::to_string(timeout_ms) + " ms");
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "stream synchronize");
    return check_err_word(b);
}

uslam_status copy_features(uslam_batch* b, const char* out_base, int frame, uslam_feature* out, int max_out, int* kept,
                           int* raw) {
    const FrameDev& F = b->frames[frame];
    const int L = b->levels;
    const uint32_t* counts = reinterpret_cast<const uint32_t*>(out_base + b->feat_off[frame]);
    int total = 0;
    for (int l = 0; l < L; ++l) {
        if (kept) kept[l] = static_cast<int>(counts[l]);
        if (raw) raw[l] = static_cast<int>(counts[L + l]);
        total += static_cast<int>(counts[l]);
    }
    if (!out) return USLAM_OK;
    if (total > max_out) return set_err(b->err(), USLAM_CAPACITY, "features: output buffer holds " + std::to_string(max_out) + " < " + std::to_string(total));
    int n = 0;
    const char* arena_out = reinterpret_cast<const char*>(b->arena + b->in_bytes);
    for (int l = 0; l < L; ++l) {
        const size_t off = reinterpret_cast<const char*>(F.feats[l]) - arena_out;
        std::memcpy(out + n, out_base + off, counts[l] * sizeof(uslam_feature));
        n += static_cast<int>(counts[l]);
    }
    return USLAM_OK;
}

uslam_status copy_matches(uslam_batch* b, const char* out_base, int pair, uslam_match* out, int max_out, int* n_out) {
    const PairDev& P = b->pairs[pair];
    const int L = b->levels;
    const char* arena_out = reinterpret_cast<const char*>(b->arena + b->in_bytes);
    const uint32_t* counts = reinterpret_cast<const uint32_t*>(out_base + b->pair_off[pair]);
    const int32_t* m = reinterpret_cast<const int32_t*>(out_base + (reinterpret_cast<const char*>(P.matches) - arena_out));
    int total = 0;
    for (int l = 0; l < L; ++l) total += static_cast<int>(std::min<uint32_t>(counts[l], P.max_matches_per_level));
    if (n_out) *n_out = total;
    if (!out) return USLAM_OK;
    if (total > max_out) return set_err(b->err(), USLAM_CAPACITY, "matches: output buffer too small");
    int n = 0;
    for (int l = 0; l < L; ++l) {
        const int c = static_cast<int>(std::min<uint32_t>(counts[l], P.max_matches_per_level));
        std::memcpy(out + n, m + static_cast<size_t>(l) * P.max_matches_per_level * 4, c * sizeof(uslam_match));
        n += c;
    }
    return USLAM_OK;
}

}  // namespace

// ====================================================================== ABI

extern "C" {

const char* uslam_status_string(uslam_status s) {
    switch (s) {
        case USLAM_OK: return "ok";
        case USLAM_INVALID_ARG: return "invalid argument";
        case USLAM_OOM: return "out of memory";
        case USLAM_TIMEOUT: return "timeout";
        case USLAM_CUDA_ERROR: return "cuda error";
        case USLAM_CAPACITY: return "capacity";
        case USLAM_NOT_READY: return "not ready";
        case USLAM_KERNEL_CHECK: return "kernel check";
    }
    return "unknown";
}

uslam_status uslam_level_dims(int width, int height, int levels, int* w_out, int* h_out) {
    if (width <= 0 || height <= 0 || levels <= 0 || levels > USLAM_MAX_LEVELS || !w_out || !h_out)
        return USLAM_INVALID_ARG;
    level_dims(width, height, levels, w_out, h_out);
    return USLAM_OK;
}

uslam_status uslam_cull_coverage(int W0, int H0, int w, int h, uint32_t* bits_out) {
    if (W0 <= 0 || H0 <= 0 || w <= 0 || h <= 0 || w > W0 || h > H0 || !bits_out) return USLAM_INVALID_ARG;
    const std::vector<uint32_t> bits = build_cull_mask(W0, H0, w, h);
    std::memcpy(bits_out, bits.data(), bits.size() * sizeof(uint32_t));
    return USLAM_OK;
}

uslam_status uslam_create(const uslam_params* params, uslam_ctx** out) {
    if (!params || !out) return USLAM_INVALID_ARG;
    *out = nullptr;
    if (params->levels < 1 || params->levels > USLAM_MAX_LEVELS || params->max_width < 1 ||
        params->max_width > kMaxWidth || params->max_height < 1 || params->max_height > 65535 ||
        params->cap_per_level < 0 || params->cap_per_level >= (1 << 24) || !params->brief_pattern ||
        (params->matcher < 0 || params->matcher > 3) ||
        ((params->matcher == 1 || params->matcher == 2) && !(params->ratio > 0.0f)) ||
        params->cell_cap < 0 || params->cell_cap > 1024 || (params->detector != 0 && params->detector != 1) ||
        params->frame_cap < 0 || params->describe_form < 0 || params->describe_form > 1)
        return USLAM_INVALID_ARG;
    auto* c = new uslam_ctx();
    c->device = params->device;
    c->levels = params->levels;
    c->max_w = params->max_width;
    c->max_h = params->max_height;
    c->cap_override = params->cap_per_level;
    // matcher 3 is matcher 0 (the same lists) with the distances from the tensor cores
    c->matcher = params->matcher == 3 ? 0 : params->matcher;
    c->win_tc = params->matcher == 3;
    c->ratio = params->ratio;
    c->cell_cap = params->cell_cap;
    c->frame_cap = params->frame_cap;
    c->describe_form = params->describe_form;
    c->detector = params->detector;
    // blur-cache margin: a rotated test point lies within ceil(radius) + 1 of
    // its keypoint (rounding of the rotation), so radius + 2 covers it.
    double rmax = 0.0;
    for (int i = 0; i < 512; ++i) {
        const double px = params->brief_pattern[2 * i], py = params->brief_pattern[2 * i + 1];
        rmax = std::max(rmax, std::sqrt(px * px + py * py));
    }
    if (rmax > 1024.0) {
        delete c;
        return USLAM_INVALID_ARG;
    }
    c->margin = static_cast<int>(std::ceil(rmax)) + 2;
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess) e = init_constants();
    if (e == cudaSuccess) e = cudaMalloc(&c->d_pattern, 1024 * sizeof(int32_t));
    if (e == cudaSuccess)
        e = cudaMemcpy(c->d_pattern, params->brief_pattern, 1024 * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (c->d_pattern) cudaFree(c->d_pattern);
        delete c;
        return e == cudaErrorMemoryAllocation ? USLAM_OOM : USLAM_CUDA_ERROR;
    }
    *out = c;
    return USLAM_OK;
}

void uslam_destroy(uslam_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    for (auto& kv : c->classes)
        for (auto* p : kv.second.d_mask) cudaFree(p);
    for (auto& kv : c->match_batches) free_batch(kv.second);
    if (c->ransac_buf) cudaFree(c->ransac_buf);
    if (c->tri_buf) cudaFree(c->tri_buf);
    if (c->d_pattern) cudaFree(c->d_pattern);
    delete c;
}

const char* uslam_last_error(const uslam_ctx* c) {
    // a copy per calling thread: valid until this thread's next call here
    thread_local std::string copy;
    copy = c ? c->err.get() : std::string("null context");
    return copy.c_str();
}

uslam_status uslam_batch_create(uslam_ctx* ctx, int n_frames, const int* widths, const int* heights, int n_pairs,
                                const int* pair_prev, const int* pair_curr, uslam_batch** out) {
    return create_batch(ctx, n_frames, widths, heights, n_pairs, pair_prev, pair_curr, false, out);
}

void uslam_batch_destroy(uslam_batch* b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    free_batch(b);
}

uslam_status uslam_batch_input_device(uslam_batch* b, int frame, uint8_t** dev_ptr, int* pitch) {
    if (!b || frame < 0 || frame >= static_cast<int>(b->frames.size()) || !dev_ptr) return USLAM_INVALID_ARG;
    *dev_ptr = const_cast<uint8_t*>(b->frames[frame].img);
    if (pitch) *pitch = b->frames[frame].img_pitch;
    return USLAM_OK;
}

uslam_status uslam_batch_input_host(uslam_batch* b, int frame, uint8_t** host_ptr, int* pitch) {
    if (!b || frame < 0 || frame >= static_cast<int>(b->frames.size()) || !host_ptr) return USLAM_INVALID_ARG;
    *host_ptr = reinterpret_cast<uint8_t*>(b->h_in + b->in_off[frame]);
    if (pitch) *pitch = b->frames[frame].img_pitch;
    return USLAM_OK;
}

uslam_status uslam_batch_set_frame(uslam_batch* b, int frame, const uint8_t* img, int pitch) {
    if (!b || frame < 0 || frame >= static_cast<int>(b->frames.size()) || !img) return USLAM_INVALID_ARG;
    const FrameDev& F = b->frames[frame];
    if (pitch < F.W0) return set_err(b->err(), USLAM_INVALID_ARG, "set_frame: pitch smaller than the frame width");
    char* dst = b->h_in + b->in_off[frame];
    for (int y = 0; y < F.H0; ++y) std::memcpy(dst + static_cast<size_t>(y) * F.img_pitch, img + static_cast<size_t>(y) * pitch, F.W0);
    return USLAM_OK;
}

uslam_status uslam_batch_upload(uslam_batch* b) {
    if (!b) return USLAM_INVALID_ARG;
    cudaError_t e = cudaMemcpyAsync(b->arena, b->h_in, b->in_bytes, cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "batch upload");
    return USLAM_OK;
}

uslam_status uslam_batch_run(uslam_batch* b) {
    if (!b) return USLAM_INVALID_ARG;
    cudaError_t e = cudaGraphLaunch(b->full.graph, b->stream);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "graph launch");
    return USLAM_OK;
}

uslam_status uslam_batch_download(uslam_batch* b) {
    if (!b) return USLAM_INVALID_ARG;
    cudaError_t e = cudaMemcpyAsync(b->h_out, b->arena + b->in_bytes, b->out_bytes, cudaMemcpyDeviceToHost, b->stream);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "batch download");
    return USLAM_OK;
}

uslam_status uslam_batch_sync(uslam_batch* b, int timeout_ms) {
    if (!b) return USLAM_INVALID_ARG;
    return sync_stream(b, timeout_ms);
}

uslam_status uslam_batch_features(uslam_batch* b, int frame, uslam_feature* out, int max_out, int* kept, int* raw) {
    if (!b || frame < 0 || frame >= static_cast<int>(b->frames.size())) return USLAM_INVALID_ARG;
    return copy_features(b, b->h_out, frame, out, max_out, kept, raw);
}

uslam_status uslam_batch_matches(uslam_batch* b, int pair, uslam_match* out, int max_out, int* n_out) {
    if (!b || pair < 0 || pair >= static_cast<int>(b->pairs.size())) return USLAM_INVALID_ARG;
    return copy_matches(b, b->h_out, pair, out, max_out, n_out);
}

uslam_status uslam_batch_pyramid_level(uslam_batch* b, int frame, int level, float* out) {
    if (!b || !out || frame < 0 || frame >= static_cast<int>(b->frames.size()) || level < 1 || level >= b->levels)
        return USLAM_INVALID_ARG;
    const FrameDev& F = b->frames[frame];
    cudaError_t e = cudaMemcpy2D(out, sizeof(float) * F.w[level], F.lvl[level], sizeof(float) * F.lvl_pitch[level],
                                 sizeof(float) * F.w[level], F.h[level], cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "pyramid readback");
    return USLAM_OK;
}

uslam_status uslam_batch_blur_level(uslam_batch* b, int frame, int level, float* out) {
    if (!b || !out || frame < 0 || frame >= static_cast<int>(b->frames.size()) || level < 0 || level >= b->levels)
        return USLAM_INVALID_ARG;
    const FrameDev& F = b->frames[frame];
    const size_t cols = static_cast<size_t>(F.w[level] + F.margin + 1);
    cudaError_t e = cudaMemcpy2D(out, sizeof(float) * cols, F.blur[level], sizeof(float) * F.bl_pitch[level],
                                 sizeof(float) * cols, static_cast<size_t>(F.h[level] + F.margin + 1),
                                 cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "blur readback");
    return USLAM_OK;
}

uslam_status uslam_blur_margin(const uslam_ctx* ctx, int* margin) {
    if (!ctx || !margin) return USLAM_INVALID_ARG;
    *margin = ctx->margin;
    return USLAM_OK;
}

uslam_status uslam_batch_keypoint_map(uslam_batch* b, int frame, int level, uint8_t* out) {
    if (!b || !out || frame < 0 || frame >= static_cast<int>(b->frames.size()) || level < 0 || level >= b->levels)
        return USLAM_INVALID_ARG;
    const FrameDev& F = b->frames[frame];
    cudaError_t e = cudaMemcpy2D(out, F.w[level], F.kpmap[level], F.kp_pitch[level], F.w[level], F.h[level],
                                 cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "keypoint map readback");
    return USLAM_OK;
}

uslam_status uslam_batch_set_stream(uslam_batch* b, void* cuda_stream) {
    if (!b) return USLAM_INVALID_ARG;
    b->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : b->own_stream;
    return USLAM_OK;
}

uslam_status uslam_batch_profile(uslam_batch* b, int iters, float* kernel_ms) {
    if (!b || iters <= 0 || !kernel_ms) return USLAM_INVALID_ARG;
    uslam_ctx* c = b->ctx;
    const Program& P = b->full;
    constexpr int K = 7;
    cudaEvent_t ev[K + 1];
    for (auto& x : ev) x = nullptr;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i <= K && e == cudaSuccess; ++i) e = cudaEventCreate(&ev[i]);
    double acc[K] = {0, 0, 0, 0, 0, 0, 0};
    const int grid = c->num_sms * 4;
    for (int it = 0; it < iters && e == cudaSuccess; ++it) {
        int k = 0;
        auto mark = [&]() {
            if (e == cudaSuccess) e = cudaEventRecord(ev[k++], b->stream);
        };
        mark();
        for (int sh = 0; sh < kNumTileShapes && e == cudaSuccess; ++sh)
            e = launch_pyramid(b->d_frames, P.tiles + P.tile_begin[sh], P.tile_begin[sh + 1] - P.tile_begin[sh], sh,
                               b->stream);
        mark();
        for (int sh = 0; sh < kNumTileShapes && e == cudaSuccess; ++sh)
            e = launch_detect(b->d_frames, P.tiles + P.tile_begin[sh], P.tile_begin[sh + 1] - P.tile_begin[sh], sh,
                              c->detector, b->d_err, b->stream);
        mark();
        if (e == cudaSuccess) e = launch_blur_border(b->d_frames, P.fsegs, P.nfsegs, grid, b->stream);
        mark();
        if (e == cudaSuccess)
            e = launch_compact_banded(b->d_frames, P.bands, P.nbands, P.fsegs, P.nfsegs, b->max_w, b->stream);
        mark();
        if (e == cudaSuccess)
            e = describe_stage(b, P, b->stream);
        mark();
        if (e == cudaSuccess && c->matcher == 0 && !b->win_tc)
            e = launch_bacc_init(b->d_frames, b->d_pairs, P.usegs, P.nusegs, b->stream);
        if (e == cudaSuccess)
            e = c->matcher == 1 ? launch_bruteforce(b->d_frames, b->d_pairs, P.psegs, P.npsegs, c->ratio, grid, b->stream)
                : c->matcher == 2
                    ? launch_bf_mma(b->d_frames, b->d_pairs, P.psegs, P.npsegs, c->ratio, c->num_sms, b->d_err, b->stream)
                : b->win_tc ? launch_win_match(b->d_frames, b->d_pairs, P.msegs, P.nmsegs, b->win_umax, P.units,
                                               c->num_sms, b->d_err, b->stream)
                    : launch_match_dyn(b->d_frames, b->d_pairs, P.msegs, P.nmsegs, c->num_sms,
                                       lane_claim(b, 0), lane_gbucket(b, 0), b->stream);
        mark();
        if (e == cudaSuccess)
            e = c->matcher != 0 ? launch_emit(b->d_frames, b->d_pairs, P.usegs, P.nusegs, b->d_err, b->stream)
                                : launch_mutual_reset(b->d_frames, b->d_pairs, P.usegs, P.nusegs, b->d_err,
                                                      lane_claim(b, 0), b->stream);
        mark();
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[K]);
        for (int q = 0; q < K && e == cudaSuccess; ++q) {
            float ms = 0.0f;
            e = cudaEventElapsedTime(&ms, ev[q], ev[q + 1]);
            acc[q] += ms;
        }
    }
    for (auto& x : ev)
        if (x) cudaEventDestroy(x);
    if (e != cudaSuccess) return c->cuda_fail(e, "profile");
    for (int q = 0; q < K; ++q) kernel_ms[q] = static_cast<float>(acc[q] / iters);
    return check_err_word(b);
}

uslam_status uslam_tile_shapes(int* n_out, int* tw, int* th) {
    if (!n_out) return USLAM_INVALID_ARG;
    *n_out = kNumTileShapes;
    for (int s = 0; s < kNumTileShapes; ++s) {
        if (tw) tw[s] = kTileShapes[s][0];
        if (th) th[s] = kTileShapes[s][1];
    }
    return USLAM_OK;
}

uslam_status uslam_set_tile_shape(uslam_ctx* ctx, int width, int height, int shape) {
    if (!ctx || width < 1 || height < 1 || shape < 0 || shape >= kNumTileShapes)
        return set_err(ctx ? &ctx->err : nullptr, USLAM_INVALID_ARG, "set_tile_shape: bad arguments");
    ctx->tile_shape[std::make_pair(width, height)] = shape;
    return USLAM_OK;
}

uslam_status uslam_get_tile_shape(const uslam_ctx* ctx, int width, int height, int* shape) {
    if (!ctx || !shape) return USLAM_INVALID_ARG;
    *shape = ctx->shape_for(width, height);
    return USLAM_OK;
}

// Autotuner: a throwaway batch of n_frames copies of the caller's frame runs
// once (pyramid masks, cull coverage), then k_pyramid + k_detect are timed
// over every frame's tiles in each shape (CUDA events on the batch stream, median of
// `reps` launches); the fastest shape is stored for the resolution class.
uslam_status uslam_autotune(uslam_ctx* ctx, int width, int height, const uint8_t* img, int pitch, int n_frames,
                            int reps, int* shape_out, float* ms_out) {
    if (!ctx || !img || n_frames < 1 || n_frames > 1024 || reps < 1 || reps > 1000 || pitch < width)
        return set_err(ctx ? &ctx->err : nullptr, USLAM_INVALID_ARG, "autotune: bad arguments");
    std::vector<int> ws(n_frames, width), hs(n_frames, height);
    uslam_batch* b = nullptr;
    uslam_status st = create_batch(ctx, n_frames, ws.data(), hs.data(), 0, nullptr, nullptr, false, &b);
    if (st != USLAM_OK) return st;
    for (int f = 0; f < n_frames && st == USLAM_OK; ++f) st = uslam_batch_set_frame(b, f, img, pitch);
    if (st == USLAM_OK) st = uslam_batch_upload(b);
    if (st == USLAM_OK) st = uslam_batch_run(b);
    if (st == USLAM_OK) st = uslam_batch_sync(b, 0);
    TileItem* d_tiles = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float best_ms = 0.0f;
    int best = -1;
    cudaError_t e = cudaSuccess;
    if (st == USLAM_OK) {
        e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
    }
    for (int s = 0; s < kNumTileShapes && st == USLAM_OK && e == cudaSuccess; ++s) {
        std::vector<TileItem> tiles;
        for (int f = 0; f < n_frames; ++f) append_tiles(&tiles, f, b->frames[f], s);
        if (d_tiles) cudaFree(d_tiles);
        d_tiles = nullptr;
        e = cudaMalloc(&d_tiles, tiles.size() * sizeof(TileItem));
        if (e == cudaSuccess)
            e = cudaMemcpy(d_tiles, tiles.data(), tiles.size() * sizeof(TileItem), cudaMemcpyHostToDevice);
        const int n = static_cast<int>(tiles.size());
        std::vector<float> t;
        for (int r = -2; r < reps && e == cudaSuccess; ++r) {
            e = cudaEventRecord(e0, b->stream);
            if (e == cudaSuccess) e = launch_pyramid(b->d_frames, d_tiles, n, s, b->stream);
            if (e == cudaSuccess) e = launch_detect(b->d_frames, d_tiles, n, s, ctx->detector, b->d_err, b->stream);
            if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (r >= 0) t.push_back(ms);  // two untimed warm-up launches
        }
        if (e != cudaSuccess) break;
        std::sort(t.begin(), t.end());
        const float med = t[t.size() / 2];
        if (ms_out) ms_out[s] = med;
        if (best < 0 || med < best_ms) {
            best = s;
            best_ms = med;
        }
    }
    if (d_tiles) cudaFree(d_tiles);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st == USLAM_OK && e != cudaSuccess) st = ctx->cuda_fail(e, "autotune");
    if (st == USLAM_OK) st = check_err_word(b);
    free_batch(b);
    if (st != USLAM_OK) return st;
    ctx->tile_shape[std::make_pair(width, height)] = best;
    if (shape_out) *shape_out = best;
    return USLAM_OK;
}

uslam_status uslam_batch_set_first_wait(uslam_batch* b, int detect_polls, int match_polls) {
    if (!b || detect_polls < -1 || match_polls < -1)
        return set_err(b ? b->err() : nullptr, USLAM_INVALID_ARG, "set_first_wait: bad arguments");
    for (FrameDev& F : b->frames) {
        F.detect_first_wait = detect_polls;
        F.match_first_wait = match_polls;
    }
    // the kernels read the frame table at run time: no new graph is needed
    cudaError_t e = cudaMemcpy(b->d_frames, b->frames.data(), sizeof(FrameDev) * b->frames.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "frame table upload");
    return USLAM_OK;
}

uslam_status uslam_batch_io_bytes(uslam_batch* b, size_t* h2d, size_t* d2h) {
    if (!b) return USLAM_INVALID_ARG;
    if (h2d) *h2d = b->in_bytes;
    if (d2h) *d2h = b->out_bytes;
    return USLAM_OK;
}

}  // extern "C"

// ================================================================= frontend

struct uslam_frontend {
    uslam_batch* b = nullptr;
    uint8_t* incoming = nullptr;  // device buffer for caller-written frames
    uint8_t* h_stage = nullptr;   // pinned u8 staging of the next host frame (H0 rows of img_pitch)
    float* h_stage_f32 = nullptr; // pinned f32 staging of the next f32 host frame (H0 rows of W0)
    float* d_f32 = nullptr;       // its device copy
    int cur = -1;                 // slot holding FeatureSet(0)
    int ref = -1;                 // slot holding FeatureSet(1)
    bool matched = false;
    // the batch's pinned output staging holds this slot's feature set / this
    // pair's matches as of their last computation (downloaded with the frame)
    bool host_frame[2] = {false, false};
    bool host_pair[2] = {false, false};
};

namespace {

// Byte range of a frame's outputs (counts + feature blocks) and of a pair's
// outputs (counts + match blocks) in the batch's outputs region.
std::pair<size_t, size_t> frame_out_range(const uslam_batch* b, int f) {
    const FrameDev& F = b->frames[f];
    const char* out0 = b->arena + b->in_bytes;
    const size_t end = static_cast<size_t>(reinterpret_cast<const char*>(F.feats[F.levels - 1]) - out0) +
                       static_cast<size_t>(std::max(F.cap, 1)) * 48;
    return {b->feat_off[f], end - b->feat_off[f]};
}
std::pair<size_t, size_t> pair_out_range(const uslam_batch* b, int p) {
    const PairDev& P = b->pairs[p];
    const char* out0 = b->arena + b->in_bytes;
    const size_t end = static_cast<size_t>(reinterpret_cast<const char*>(P.matches) - out0) +
                       static_cast<size_t>(b->levels) * std::max(P.max_matches_per_level, 1) * 16;
    return {b->pair_off[p], end - b->pair_off[p]};
}

// Choose the slot of the next frame and enqueue its copy and work.
// src_host (u8) or src_f32 (f32 in [0, 1]) != NULL: the frame goes through
// the pinned staging (an asynchronous H2D copy); else src_dev != NULL: D2D
// from caller device memory; else D2D from `incoming`.  download: the new
// feature set and matches are copied back into the pinned output staging
// behind the work, for the feature / match getters.
uslam_status frontend_enqueue(uslam_frontend* fe, const uint8_t* src_host, const float* src_f32,
                              const uint8_t* src_dev, int pitch, int advance_reference, bool download,
                              int* matched) {
    uslam_batch* b = fe->b;
    const FrameDev& F0 = b->frames[0];
    // LoadDataCPUPass::shiftFeatureSets (load_features_cpu.cpp:111-142): the
    // current set becomes the reference when asked or when none exists yet;
    // otherwise the reference is kept and the current set is replaced.
    if ((src_host || src_f32 || src_dev) && pitch < F0.W0)
        return set_err(b->err(), USLAM_INVALID_ARG, "process: pitch smaller than the frame width");
    int slot;
    if (fe->cur < 0) {
        slot = 0;
    } else {
        if (fe->ref < 0 || advance_reference) fe->ref = fe->cur;
        slot = 1 - fe->ref;
    }
    uint8_t* dst = const_cast<uint8_t*>(b->frames[slot].img);
    const size_t frame_bytes = static_cast<size_t>(F0.H0) * F0.img_pitch;
    cudaError_t e;
    if (src_host) {
        // the previous frame's upload from the staging has completed: every
        // host-frame call returns after its work (and its copies) finished
        for (int y = 0; y < F0.H0; ++y)
            std::memcpy(fe->h_stage + static_cast<size_t>(y) * F0.img_pitch, src_host + static_cast<size_t>(y) * pitch,
                        F0.W0);
        e = cudaMemcpyAsync(dst, fe->h_stage, frame_bytes, cudaMemcpyHostToDevice, b->stream);
    } else if (src_f32) {
        // f32 rows into the pinned f32 staging, one asynchronous copy, the
        // bytes recovered on the device
        const size_t row_bytes = sizeof(float) * F0.W0;
        for (int y = 0; y < F0.H0; ++y)
            std::memcpy(fe->h_stage_f32 + static_cast<size_t>(y) * F0.W0, src_f32 + static_cast<size_t>(y) * pitch,
                        row_bytes);
        e = cudaMemcpyAsync(fe->d_f32, fe->h_stage_f32, row_bytes * F0.H0, cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess) e = launch_frame_from_f32(fe->d_f32, F0.W0, F0.H0, dst, F0.img_pitch, b->stream);
    } else if (src_dev) {
        e = cudaMemcpy2DAsync(dst, F0.img_pitch, src_dev, pitch, F0.W0, F0.H0, cudaMemcpyDeviceToDevice, b->stream);
    } else {
        e = cudaMemcpyAsync(dst, fe->incoming, frame_bytes, cudaMemcpyDeviceToDevice, b->stream);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_err, 0, sizeof(uint32_t), b->stream);
    if (e == cudaSuccess) e = enqueue_program(b, b->frame_prog[slot]);
    fe->cur = slot;
    fe->matched = false;
    fe->host_frame[slot] = false;
    const int pair = slot == 0 ? 0 : 1;  // pair 0 = slot1 -> slot0, pair 1 = slot0 -> slot1
    if (e == cudaSuccess && fe->ref >= 0) {
        fe->host_pair[pair] = false;
        e = enqueue_program(b, b->pair_prog[pair]);
        fe->matched = true;
    }
    if (e == cudaSuccess && download) {
        const auto fr = frame_out_range(b, slot);
        e = cudaMemcpyAsync(b->h_out + fr.first, b->arena + b->in_bytes + fr.first, fr.second,
                            cudaMemcpyDeviceToHost, b->stream);
        if (e == cudaSuccess && fe->matched) {
            const auto pr = pair_out_range(b, pair);
            e = cudaMemcpyAsync(b->h_out + pr.first, b->arena + b->in_bytes + pr.first, pr.second,
                                cudaMemcpyDeviceToHost, b->stream);
        }
    }
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "frontend launch");
    if (matched) *matched = fe->matched ? 1 : 0;
    return USLAM_OK;
}

// A synchronous host-frame call: enqueue with the download, wait, and mark
// the downloaded outputs current.
uslam_status frontend_process_host(uslam_frontend* fe, const uint8_t* img, const float* img_f32, int pitch,
                                   int advance_reference) {
    int matched = 0;
    uslam_status s = frontend_enqueue(fe, img, img_f32, nullptr, pitch, advance_reference, true, &matched);
    if (s != USLAM_OK) return s;
    s = sync_stream(fe->b, 0);
    if (s != USLAM_OK) return s;
    fe->host_frame[fe->cur] = true;
    if (matched) fe->host_pair[fe->cur == 0 ? 0 : 1] = true;
    return matched ? USLAM_OK : USLAM_NOT_READY;
}

// Bring the whole outputs region to the pinned staging (after asynchronous
// enqueues, whose outputs were not downloaded).
uslam_status frontend_refresh(uslam_frontend* fe) {
    uslam_batch* b = fe->b;
    cudaError_t e = cudaMemcpy(b->h_out, b->arena + b->in_bytes, b->out_bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return b->ctx->cuda_fail(e, "outputs readback");
    fe->host_frame[0] = fe->host_frame[1] = fe->host_pair[0] = fe->host_pair[1] = true;
    return USLAM_OK;
}

}  // namespace

extern "C" {

uslam_status uslam_frontend_create(uslam_ctx* ctx, int width, int height, uslam_frontend** out) {
    if (!ctx || !out) return USLAM_INVALID_ARG;
    const int ws[2] = {width, width}, hs[2] = {height, height};
    const int prev[2] = {1, 0}, curr[2] = {0, 1};  // pair 0: slot1 -> slot0, pair 1: slot0 -> slot1
    uslam_batch* b = nullptr;
    uslam_status s = create_batch(ctx, 2, ws, hs, 2, prev, curr, true, &b, true);
    if (s != USLAM_OK) return s;
    auto* fe = new uslam_frontend();
    fe->b = b;
    const size_t frame_bytes = static_cast<size_t>(b->frames[0].H0) * b->frames[0].img_pitch;
    const size_t f32_bytes = sizeof(float) * static_cast<size_t>(b->frames[0].H0) * b->frames[0].W0;
    cudaError_t e = cudaMalloc(&fe->incoming, frame_bytes);
    if (e == cudaSuccess) e = cudaHostAlloc(&fe->h_stage, frame_bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc(&fe->h_stage_f32, f32_bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc(&fe->d_f32, f32_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (fe->incoming) cudaFree(fe->incoming);
        if (fe->h_stage) cudaFreeHost(fe->h_stage);
        if (fe->h_stage_f32) cudaFreeHost(fe->h_stage_f32);
        if (fe->d_f32) cudaFree(fe->d_f32);
        uslam_batch_destroy(b);
        delete fe;
        return set_err(&ctx->err, USLAM_OOM, "frontend input buffer allocation refused");
    }
    std::memset(fe->h_stage, 0, frame_bytes);
    *out = fe;
    return USLAM_OK;
}

void uslam_frontend_destroy(uslam_frontend* fe) {
    if (!fe) return;
    cudaSetDevice(fe->b->ctx->device);
    if (fe->incoming) cudaFree(fe->incoming);
    if (fe->h_stage) cudaFreeHost(fe->h_stage);
    if (fe->h_stage_f32) cudaFreeHost(fe->h_stage_f32);
    if (fe->d_f32) cudaFree(fe->d_f32);
    uslam_batch_destroy(fe->b);
    delete fe;
}

uslam_status uslam_frontend_input_device(uslam_frontend* fe, uint8_t** dev_ptr, int* pitch) {
    if (!fe || !dev_ptr) return USLAM_INVALID_ARG;
    *dev_ptr = fe->incoming;
    if (pitch) *pitch = fe->b->frames[0].img_pitch;
    return USLAM_OK;
}

uslam_status uslam_frontend_enqueue(uslam_frontend* fe, const uint8_t* dev_img, int pitch, int advance_reference,
                                    int* matched) {
    if (!fe) return USLAM_INVALID_ARG;
    return frontend_enqueue(fe, nullptr, nullptr, dev_img, pitch, advance_reference, false, matched);
}

uslam_status uslam_frontend_sync(uslam_frontend* fe) {
    if (!fe) return USLAM_INVALID_ARG;
    return sync_stream(fe->b, 0);
}

uslam_status uslam_frontend_process(uslam_frontend* fe, const uint8_t* img, int pitch, int advance_reference) {
    if (!fe) return USLAM_INVALID_ARG;
    if (!img) {
        // the frame is already in the frontend's device input buffer
        int matched = 0;
        uslam_status s = frontend_enqueue(fe, nullptr, nullptr, nullptr, pitch, advance_reference, true, &matched);
        if (s != USLAM_OK) return s;
        s = sync_stream(fe->b, 0);
        if (s != USLAM_OK) return s;
        fe->host_frame[fe->cur] = true;
        if (matched) fe->host_pair[fe->cur == 0 ? 0 : 1] = true;
        return matched ? USLAM_OK : USLAM_NOT_READY;
    }
    return frontend_process_host(fe, img, nullptr, pitch, advance_reference);
}

uslam_status uslam_frontend_process_f32(uslam_frontend* fe, const float* img, int pitch, int advance_reference) {
    if (!fe || !img) return USLAM_INVALID_ARG;
    return frontend_process_host(fe, nullptr, img, pitch, advance_reference);
}

uslam_status uslam_frontend_features(uslam_frontend* fe, int which, uslam_feature* out, int max_out, int* kept,
                                     int* raw) {
    if (!fe || (which != 0 && which != 1)) return USLAM_INVALID_ARG;
    const int slot = which == 0 ? fe->cur : fe->ref;
    if (slot < 0) return set_err(fe->b->err(), USLAM_NOT_READY, "features: that feature set does not exist yet");
    if (!fe->host_frame[slot]) {
        const uslam_status s = frontend_refresh(fe);
        if (s != USLAM_OK) return s;
    }
    return copy_features(fe->b, fe->b->h_out, slot, out, max_out, kept, raw);
}

uslam_status uslam_frontend_matches(uslam_frontend* fe, uslam_match* out, int max_out, int* n_out) {
    if (!fe) return USLAM_INVALID_ARG;
    if (!fe->matched) return set_err(fe->b->err(), USLAM_NOT_READY, "matches: no reference feature set yet");
    const int pair = fe->cur == 0 ? 0 : 1;
    if (!fe->host_pair[pair]) {
        const uslam_status s = frontend_refresh(fe);
        if (s != USLAM_OK) return s;
    }
    return copy_matches(fe->b, fe->b->h_out, pair, out, max_out, n_out);
}

}  // extern "C"

// ============================================================ feature sets
// The single-frame export set: a device-resident feature set, one-shot detect
// + describe into it, and a match between two sets.

struct uslam_featset {
    uslam_ctx* ctx = nullptr;
    uslam_batch* b = nullptr;  // one frame, no pairs
    int W = 0, H = 0;
    bool valid = false;
};

namespace {

// Copy frame 0 of a one-frame batch (feature blocks, counts and the matcher's
// lists) into frame `slot` of a batch of the same frame size.
cudaError_t copy_frame_state(const uslam_batch* src, uslam_batch* dst, int slot, cudaStream_t st) {
    const FrameDev& A = src->frames[0];
    const FrameDev& B = dst->frames[slot];
    const size_t capa = static_cast<size_t>(std::max(A.cap, 1));
    cudaError_t e = cudaMemcpyAsync(B.kept, A.kept, 2 * sizeof(uint32_t) * A.levels, cudaMemcpyDeviceToDevice, st);
    for (int l = 0; l < A.levels && e == cudaSuccess; ++l) {
        const size_t cols = USLAM_MATCH_BANDS * (static_cast<size_t>(A.w[l]) + 1) + USLAM_MATCH_BANDS + 1;
        e = cudaMemcpyAsync(B.feats[l], A.feats[l], capa * 48, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(B.xorder[l], A.xorder[l], USLAM_MATCH_BANDS * capa * 4, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.colstart[l], A.colstart[l], cols * 4, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.qorder[l], A.qorder[l], capa * 4, cudaMemcpyDeviceToDevice, st);
    }
    if (A.bf8 && B.bf8 && e == cudaSuccess) {
        const size_t rows = tc_rows(A);
        e = cudaMemcpyAsync(B.bf8, A.bf8, rows * 256, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.bfext, A.bfext, rows * 32, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.bfpop, A.bfpop, rows * 4, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.bfid, A.bfid, rows * 4, cudaMemcpyDeviceToDevice, st);
    }
    if (A.wq8 && B.wq8 && e == cudaSuccess) {
        // the windowed tensor-core matcher's operand rows (same frame size,
        // so the same row strides)
        const size_t qrows = static_cast<size_t>(A.levels) * A.wq_rows;
        const size_t crows = static_cast<size_t>(A.levels) * USLAM_MATCH_BANDS * A.wc_rows;
        e = cudaMemcpyAsync(B.wq8, A.wq8, qrows * 256, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.wc8, A.wc8, crows * 256, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.wcext, A.wcext, crows * 32, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.wcy, A.wcy, crows * 2, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(B.wcid, A.wcid, crows * 4, cudaMemcpyDeviceToDevice, st);
    }
    return e;
}

}  // namespace

extern "C" {

uslam_status uslam_featset_create(uslam_ctx* ctx, int width, int height, uslam_featset** out) {
    if (!ctx || !out) return USLAM_INVALID_ARG;
    uslam_batch* b = nullptr;
    uslam_status s = create_batch(ctx, 1, &width, &height, 0, nullptr, nullptr, false, &b, true);
    if (s != USLAM_OK) return s;
    auto* fs = new uslam_featset();
    fs->ctx = ctx;
    fs->b = b;
    fs->W = width;
    fs->H = height;
    *out = fs;
    return USLAM_OK;
}

void uslam_featset_destroy(uslam_featset* fs) {
    if (!fs) return;
    free_batch(fs->b);
    delete fs;
}

uslam_status uslam_detect_describe(uslam_ctx* ctx, const uint8_t* img, int width, int height, int pitch,
                                   uslam_featset* out) {
    if (!ctx || !img || !out || out->ctx != ctx) return USLAM_INVALID_ARG;
    if (width != out->W || height != out->H)
        return set_err(&ctx->err, USLAM_INVALID_ARG, "detect_describe: frame size differs from the feature set's");
    uslam_status s = uslam_batch_set_frame(out->b, 0, img, pitch);
    if (s == USLAM_OK) s = uslam_batch_upload(out->b);
    if (s == USLAM_OK) s = uslam_batch_run(out->b);
    if (s == USLAM_OK) s = uslam_batch_sync(out->b, 0);
    out->valid = s == USLAM_OK;
    return s;
}

uslam_status uslam_detect_describe_f32(uslam_ctx* ctx, const float* img, int width, int height, int pitch,
                                       uslam_featset* out) {
    if (!ctx || !img || !out || out->ctx != ctx || pitch < width || width < 1 || height < 1)
        return USLAM_INVALID_ARG;
    if (width != out->W || height != out->H)
        return set_err(&ctx->err, USLAM_INVALID_ARG, "detect_describe_f32: frame size differs from the feature set's");
    // f32 pixels in [0, 1] (the reference's FrameBW, u8 / 255) back to u8:
    // exact for u8 / 255 values, others round to the nearest step
    uint8_t* host = nullptr;
    int hp = 0;
    uslam_status s = uslam_batch_input_host(out->b, 0, &host, &hp);
    if (s != USLAM_OK) return s;
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            const float v = img[static_cast<size_t>(y) * pitch + x] * 255.0f;
            host[static_cast<size_t>(y) * hp + x] = static_cast<uint8_t>(std::lrint(std::min(std::max(v, 0.0f), 255.0f)));
        }
    s = uslam_batch_upload(out->b);
    if (s == USLAM_OK) s = uslam_batch_run(out->b);
    if (s == USLAM_OK) s = uslam_batch_sync(out->b, 0);
    out->valid = s == USLAM_OK;
    return s;
}

uslam_status uslam_featset_features(uslam_featset* fs, uslam_feature* out, int max_out, int* kept, int* raw) {
    if (!fs) return USLAM_INVALID_ARG;
    if (!fs->valid) return set_err(&fs->ctx->err, USLAM_NOT_READY, "featset_features: nothing detected yet");
    uslam_status s = uslam_batch_download(fs->b);
    if (s == USLAM_OK) s = uslam_batch_sync(fs->b, 0);
    if (s == USLAM_OK) s = uslam_batch_features(fs->b, 0, out, max_out, kept, raw);
    return s;
}

uslam_status uslam_match_sets(uslam_ctx* ctx, const uslam_featset* prev, const uslam_featset* curr, uslam_match* out,
                              int max_out, int* n_out) {
    if (!ctx || !prev || !curr || !n_out || prev->ctx != ctx || curr->ctx != ctx) return USLAM_INVALID_ARG;
    if (!prev->valid || !curr->valid) return set_err(&ctx->err, USLAM_NOT_READY, "match: a feature set is empty");
    if (prev->W != curr->W || prev->H != curr->H)
        return set_err(&ctx->err, USLAM_INVALID_ARG, "match: the feature sets come from frames of different sizes");
    const auto key = std::make_pair(prev->W, prev->H);
    auto it = ctx->match_batches.find(key);
    if (it == ctx->match_batches.end()) {
        const int ws[2] = {prev->W, prev->W}, hs[2] = {prev->H, prev->H};
        const int pp = 0, pc = 1;
        uslam_batch* mb = nullptr;
        uslam_status s = create_batch(ctx, 2, ws, hs, 1, &pp, &pc, true, &mb, true);
        if (s != USLAM_OK) return s;
        it = ctx->match_batches.emplace(key, mb).first;
    }
    uslam_batch* mb = it->second;
    // the sets' last work is complete (detect_describe synchronises); the
    // copies and the match run on the match batch's stream
    cudaError_t e = copy_frame_state(prev->b, mb, 0, mb->stream);
    if (e == cudaSuccess) e = copy_frame_state(curr->b, mb, 1, mb->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(mb->d_err, 0, sizeof(uint32_t), mb->stream);
    if (e == cudaSuccess) e = enqueue_program(mb, mb->pair_prog[0]);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "match");
    uslam_status s = uslam_batch_download(mb);
    if (s == USLAM_OK) s = uslam_batch_sync(mb, 0);
    if (s == USLAM_OK) s = uslam_batch_matches(mb, 0, out, max_out, n_out);
    return s;
}

}  // extern "C"

namespace uslam_rt {

namespace {
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        cudaGetLastError();
    });
    return fn;
}
}  // namespace

uslam_status encode_tile_maps(const FrameDev& F, int detector, void* out, ErrText* err) {
    static_assert(sizeof(CUtensorMap) == USLAM_TMAP_BYTES, "tensor map size");
    const EncodeTiledFn fn = encode_tiled();
    if (!fn) return set_err(err, USLAM_CUDA_ERROR, "cuTensorMapEncodeTiled is not available from the driver");
    const int hy = detector == 1 ? USLAM_TILE_HY_CFG : USLAM_TILE_HY;
    for (int l = 0; l < F.levels; ++l)
        for (int sh = 0; sh < kNumTileShapes; ++sh) {
            CUtensorMap* m =
                reinterpret_cast<CUtensorMap*>(static_cast<char*>(out) +
                                               (static_cast<size_t>(l) * USLAM_TMAPS_PER_LEVEL + sh) * USLAM_TMAP_BYTES);
            const cuuint64_t dims[2] = {static_cast<cuuint64_t>(F.w[l]), static_cast<cuuint64_t>(F.h[l])};
            const cuuint64_t strides[1] = {static_cast<cuuint64_t>(F.lvl_pitch[l]) * 4u};
            const cuuint32_t box[2] = {static_cast<cuuint32_t>(kTileShapes[sh][0] + 2 * USLAM_TILE_XPAD),
                                       static_cast<cuuint32_t>(kTileShapes[sh][1] + 2 * hy)};
            const cuuint32_t estr[2] = {1u, 1u};
            const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, F.lvl[l], dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS)
                return set_err(err, USLAM_CUDA_ERROR,
                               "tensor map encode failed (level " + std::to_string(l) + ", shape " + std::to_string(sh) +
                                   ", code " + std::to_string(static_cast<int>(r)) + ")");
        }
    // the blur caches, for k_describe_tiled: box = a describe item's chunk
    // (KDT_CW columns, 32 rows) widened by RX columns and R rows each side
    if (uslam::describe_tiled_smem(F.margin) == 0) return USLAM_OK;
    const int R = F.margin - 1, RX = (R + 3) & ~3;
    for (int l = 0; l < F.levels; ++l) {
        CUtensorMap* m = reinterpret_cast<CUtensorMap*>(
            static_cast<char*>(out) + (static_cast<size_t>(l) * USLAM_TMAPS_PER_LEVEL + kNumTileShapes) * USLAM_TMAP_BYTES);
        const cuuint64_t dims[2] = {static_cast<cuuint64_t>(F.w[l] + F.margin + 1),
                                    static_cast<cuuint64_t>(F.h[l] + F.margin + 1)};
        const cuuint64_t strides[1] = {static_cast<cuuint64_t>(F.bl_pitch[l]) * 4u};
        const cuuint32_t box[2] = {static_cast<cuuint32_t>(KDT_CW + 2 * RX), static_cast<cuuint32_t>(32 + 2 * R)};
        const cuuint32_t estr[2] = {1u, 1u};
        const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, F.blur[l], dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return set_err(err, USLAM_CUDA_ERROR,
                           "blur-cache tensor map encode failed (level " + std::to_string(l) + ", code " +
                               std::to_string(static_cast<int>(r)) + ")");
    }
    return USLAM_OK;
}

}  // namespace uslam_rt
