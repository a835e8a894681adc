// noalloc.cu — a matcher entry point that performs no device allocation.
//
// Some callers of this library cannot call cudaMalloc at the moment they
// need a match: a host runtime that hands out device memory only from its own
// pool, a real-time loop that must not take the allocator's locks or risk an
// allocation failure mid-frame, or code running where the CUDA context is
// shared and its memory budget is fixed in advance.  uslam_match_noalloc
// serves them: the caller passes the two feature sets and the output buffers
// (all device memory it already owns), and every piece of scratch the match
// needs lives in one file-scope __device__ array of fixed size, which every
// GPU that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/uslam.h"
#include "uslam_internal.h"

namespace uslam {
struct MatchSegDev {
    int pair;
    int dir;
    int level;
};
cudaError_t launch_match(const FrameDev*, const PairDev*, const void*, int, int, cudaStream_t);
cudaError_t launch_mutual(const FrameDev*, const PairDev*, const SegDev*, int, uint32_t*, cudaStream_t);
cudaError_t launch_bacc_init(const FrameDev*, const PairDev*, const SegDev*, int, cudaStream_t);
cudaError_t launch_xsort(const FrameDev*, const SegDev*, int, int, cudaStream_t);
cudaError_t set_compact_smem(int max_w);
}  // namespace uslam

using namespace uslam;

namespace {

constexpr size_t kNoallocScratchBytes = size_t(4) << 20;  // 4 MiB per device
constexpr int kMaxDevices = 64;

// The no-alloc matcher's scratch.  Host code must not use this name as an
// address: it is a host-side stand-in.  The device address comes from
// cudaGetSymbolAddress once per device and CUDA context (see
// scratch_for_device).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Everything the match kernels read besides the features, written into the
// scratch by one small kernel that receives it by value (no host copy).
struct NoallocTables {
    FrameDev frames[2];
    PairDev pair;
    MatchSegDev msegs[USLAM_MAX_LEVELS];
    SegDev usegs[USLAM_MAX_LEVELS];
    SegDev xsegs[2 * USLAM_MAX_LEVELS];
    uint32_t counts[2][2 * USLAM_MAX_LEVELS];  // per frame: kept[levels], raw[levels]
};

__global__ void k_noalloc_tables(const NoallocTables t, NoallocTables* dst) {
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&t);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    for (size_t i = threadIdx.x; i < sizeof(NoallocTables) / 4; i += blockDim.x) d[i] = s[i];
}

// The caller's feature records are device memory the host cannot check, and
// the x-sort indexes its shared histogram by x: every record's x and y must be
// integers (as f32) inside its level.  A record that is not (NaN included)
// sets USLAM_ERR_BAD_RECORD in *bad; k_noalloc_gate then empties both sets, so
// the sort and the match that follow on the stream see no features, and the
// host returns USLAM_INVALID_ARG after its one synchronisation.
constexpr uint32_t USLAM_ERR_BAD_RECORD = 1u << 16;

__global__ void k_noalloc_validate(const NoallocTables* t, uint32_t* bad) {
    for (int f = 0; f < 2; ++f) {
        const FrameDev& F = t->frames[f];
        for (int l = 0; l < F.levels; ++l) {
            const uint32_t n = F.kept[l];
            const uint32_t* rec = F.feats[l];
            const float w = (float)F.w[l], h = (float)F.h[l];
            for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
                const float x = __uint_as_float(rec[(size_t)i * 12u]);
                const float y = __uint_as_float(rec[(size_t)i * 12u + 1u]);
                const bool ok = x >= 0.0f && x < w && y >= 0.0f && y < h && x == truncf(x) && y == truncf(y);
                if (!ok) atomicOr(bad, USLAM_ERR_BAD_RECORD);
            }
        }
    }
}

// After k_noalloc_validate: a bad record empties both feature sets.
__global__ void k_noalloc_gate(NoallocTables* t, const uint32_t* err) {
    if (!(*err & USLAM_ERR_BAD_RECORD)) return;
    for (int i = threadIdx.x; i < 2 * 2 * USLAM_MAX_LEVELS; i += blockDim.x) (&t->counts[0][0])[i] = 0u;
}

struct DeviceScratch {
    unsigned char* ptr = nullptr;
    int num_sms = 0;
    void* context = nullptr;  // the CUDA context the address belongs to
};

std::mutex g_setup_mutex;
DeviceScratch g_scratch_by_device[kMaxDevices];

// The current CUDA context, read through the driver entry point (the runtime
// has no call for it); a reset device gets a new context, and the module that
// holds the scratch array is loaded again, possibly at another address.
using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        cudaGetLastError();
        return reinterpret_cast<CtxGetCurrentFn>(p);
    }();
    return fn;
}

// Set-up, once per device and CUDA context, with that device current: the
// scratch's device address (cudaGetSymbolAddress) and the SM count.  It runs
// on the first call on a device, and again on the first call after the
// device's context was reset.
cudaError_t scratch_for_device(int device, DeviceScratch* out) {
    void* cur = nullptr;
    const CtxGetCurrentFn get = ctx_get_current();
    if (!get || get(&cur) != 0 || !cur) return cudaErrorInitializationError;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceScratch& d = g_scratch_by_device[device];
    if (d.context != cur) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        e = cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess) return e;
        d.ptr = static_cast<unsigned char*>(p);
        d.context = cur;
    }
    *out = d;
    return cudaSuccess;
}

// Makes `device` current for the call and puts the caller's device back.
struct DeviceGuard {
    int prev = -1;
    cudaError_t set(int device) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) {
            prev = -1;
            return e;
        }
        return prev == device ? cudaSuccess : cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int now = -1;
        if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
    }
};

uslam_status fail(char* err, size_t err_len, uslam_status s, const char* msg) {
    if (err && err_len > 0) std::snprintf(err, err_len, "%s", msg);
    return s;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

extern "C" uslam_status uslam_match_noalloc(int device, int width, int height, int levels,
                                            const uslam_feature* prev_feats, const int* prev_kept,
                                            const uslam_feature* curr_feats, const int* curr_kept, uslam_match* out,
                                            uint32_t* out_counts, int out_cap_per_level, void* stream, char* err,
                                            size_t err_len) {
    if (device < 0 || device >= kMaxDevices || width <= 0 || height <= 0 || width > 12000 || levels < 1 ||
        levels > USLAM_MAX_LEVELS || !prev_kept || !curr_kept || !out || !out_counts || out_cap_per_level < 1)
        return fail(err, err_len, USLAM_INVALID_ARG, "match_noalloc: bad arguments");
    int wl[USLAM_MAX_LEVELS], hl[USLAM_MAX_LEVELS];
    if (uslam_level_dims(width, height, levels, wl, hl) != USLAM_OK)
        return fail(err, err_len, USLAM_INVALID_ARG, "match_noalloc: bad frame size");
    for (int l = 0; l < levels; ++l)
        if (wl[l] < 1 || hl[l] < 1) return fail(err, err_len, USLAM_INVALID_ARG, "match_noalloc: empty pyramid level");
    const int* kept[2] = {prev_kept, curr_kept};
    const uslam_feature* feats[2] = {prev_feats, curr_feats};
    int cap[2] = {1, 1};
    long long total[2] = {0, 0};
    for (int f = 0; f < 2; ++f) {
        for (int l = 0; l < levels; ++l) {
            if (kept[f][l] < 0 || kept[f][l] >= (1 << 24))
                return fail(err, err_len, USLAM_INVALID_ARG, "match_noalloc: feature count out of range");
            cap[f] = std::max(cap[f], kept[f][l]);
            total[f] += kept[f][l];
        }
        if (total[f] > 0 && !feats[f]) return fail(err, err_len, USLAM_INVALID_ARG, "match_noalloc: null features");
        // the matcher reads each record's descriptor as two 16-byte vectors
        if (total[f] > 0 && reinterpret_cast<uintptr_t>(feats[f]) % 16u != 0u)
            return fail(err, err_len, USLAM_INVALID_ARG, "match_noalloc: feature records not 16-byte aligned");
    }
    if (reinterpret_cast<uintptr_t>(out) % 4u != 0u || reinterpret_cast<uintptr_t>(out_counts) % 4u != 0u)
        return fail(err, err_len, USLAM_INVALID_ARG, "match_noalloc: output buffers not 4-byte aligned");
    if (out_cap_per_level < cap[0])
        return fail(err, err_len, USLAM_INVALID_ARG, "match_noalloc: out_cap_per_level below the previous set's largest level");

    // scratch layout: [tables][xorder, qorder f0][xorder, qorder f1][colstart f0][colstart f1][a2b][b -> a
    // accumulators][error]
    // (per level: USLAM_MATCH_BANDS candidate lists of cap entries, the query order, and per band
    // the column table, then the band offsets)
    size_t cur = align256(sizeof(NoallocTables));
    size_t xorder_off[2], qorder_off[2], colstart_off[2];
    for (int f = 0; f < 2; ++f) {
        xorder_off[f] = cur;
        cur = align256(cur + sizeof(uint32_t) * USLAM_MATCH_BANDS * static_cast<size_t>(levels) * cap[f]);
        qorder_off[f] = cur;
        cur = align256(cur + sizeof(uint32_t) * static_cast<size_t>(levels) * cap[f]);
    }
    size_t colsum = 0;
    for (int l = 0; l < levels; ++l) colsum += USLAM_MATCH_BANDS * (static_cast<size_t>(wl[l]) + 1) + USLAM_MATCH_BANDS + 1;
    for (int f = 0; f < 2; ++f) {
        colstart_off[f] = cur;
        cur = align256(cur + sizeof(uint32_t) * colsum);
    }
    const size_t a2b_off = cur;
    cur = align256(cur + sizeof(int32_t) * static_cast<size_t>(levels) * cap[0]);
    const size_t bacc_off = cur;
    cur = align256(cur + 16u * static_cast<size_t>(levels) * cap[1]);
    const size_t err_off = cur;
    cur += 256;
    if (cur > kNoallocScratchBytes) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "match_noalloc: needs %zu bytes of scratch, the fixed maximum is %zu", cur,
                      kNoallocScratchBytes);
        return fail(err, err_len, USLAM_CAPACITY, msg);
    }

    DeviceGuard guard;
    cudaError_t e = guard.set(device);
    DeviceScratch ds;
    if (e == cudaSuccess) e = scratch_for_device(device, &ds);
    if (e != cudaSuccess) return fail(err, err_len, USLAM_CUDA_ERROR, cudaGetErrorString(e));
    unsigned char* base = ds.ptr;
    auto* dtab = reinterpret_cast<NoallocTables*>(base);

    NoallocTables t;
    std::memset(&t, 0, sizeof t);
    for (int f = 0; f < 2; ++f) {
        FrameDev& F = t.frames[f];
        F.W0 = width;
        F.H0 = height;
        F.levels = levels;
        F.cap = cap[f];
        F.kept = reinterpret_cast<uint32_t*>(base + offsetof(NoallocTables, counts)) + f * 2 * USLAM_MAX_LEVELS;
        F.raw = F.kept + levels;
        size_t foff = 0, coff = 0;
        for (int l = 0; l < levels; ++l) {
            F.w[l] = wl[l];
            F.h[l] = hl[l];
            F.feats[l] = reinterpret_cast<uint32_t*>(const_cast<uslam_feature*>(feats[f]) + foff);
            F.xorder[l] = reinterpret_cast<uint32_t*>(base + xorder_off[f]) +
                          static_cast<size_t>(l) * USLAM_MATCH_BANDS * cap[f];
            F.qorder[l] = reinterpret_cast<uint32_t*>(base + qorder_off[f]) + static_cast<size_t>(l) * cap[f];
            F.colstart[l] = reinterpret_cast<uint32_t*>(base + colstart_off[f]) + coff;
            t.counts[f][l] = static_cast<uint32_t>(kept[f][l]);
            t.counts[f][levels + l] = static_cast<uint32_t>(kept[f][l]);
            foff += static_cast<size_t>(kept[f][l]);
            coff += USLAM_MATCH_BANDS * (static_cast<size_t>(wl[l]) + 1) + USLAM_MATCH_BANDS + 1;
            t.xsegs[f * levels + l] = SegDev{f, l};
        }
    }
    PairDev& P = t.pair;
    P.prev = 0;
    P.curr = 1;
    P.a2b = reinterpret_cast<int32_t*>(base + a2b_off);
    P.bacc = reinterpret_cast<uint4*>(base + bacc_off);
    P.matches = reinterpret_cast<int32_t*>(out);
    P.match_count = out_counts;
    P.max_matches_per_level = out_cap_per_level;
    // match_features_cpu.cpp:76-77: 0.1F * frame size, in f32
    P.max_dx = 0.1f * static_cast<float>(static_cast<uint32_t>(width));
    P.max_dy = 0.1f * static_cast<float>(static_cast<uint32_t>(height));
    for (int l = 0; l < levels; ++l) {
        t.msegs[l] = MatchSegDev{0, 1, l};  // both directions from the previous set's queries
        t.usegs[l] = SegDev{0, l};
    }

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* derr = reinterpret_cast<uint32_t*>(base + err_off);
    int max_w = 1;
    for (int l = 0; l < levels; ++l) max_w = std::max(max_w, wl[l]);
    k_noalloc_tables<<<1, 256, 0, st>>>(t, dtab);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemsetAsync(derr, 0, sizeof(uint32_t), st);  // the error word must start at zero
    if (e == cudaSuccess && (total[0] > 0 || total[1] > 0)) {
        k_noalloc_validate<<<ds.num_sms, 256, 0, st>>>(dtab, derr);
        e = cudaGetLastError();
        if (e == cudaSuccess) {
            k_noalloc_gate<<<1, 64, 0, st>>>(dtab, derr);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        e = set_compact_smem(max_w);  // a function attribute, not an allocation
        if (e == cudaSuccess) e = launch_xsort(dtab->frames, dtab->xsegs, 2 * levels, max_w, st);
    }
    if (e == cudaSuccess) e = launch_bacc_init(dtab->frames, &dtab->pair, dtab->usegs, levels, st);
    if (e == cudaSuccess) e = launch_match(dtab->frames, &dtab->pair, dtab->msegs, levels, ds.num_sms, st);
    if (e == cudaSuccess) e = launch_mutual(dtab->frames, &dtab->pair, dtab->usegs, levels, derr, st);
    uint32_t word = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&word, derr, sizeof word, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(err, err_len, USLAM_CUDA_ERROR, cudaGetErrorString(e));
    if (word & USLAM_ERR_BAD_RECORD)
        return fail(err, err_len, USLAM_INVALID_ARG,
                    "match_noalloc: a feature record's x or y is not an integer inside its level");
    if (word != 0u) return fail(err, err_len, USLAM_KERNEL_CHECK, "match_noalloc: match list overflow");
    if (err && err_len > 0) err[0] = '\0';
    return USLAM_OK;
}
