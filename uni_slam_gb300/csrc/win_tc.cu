// win_tc.cu — the reference's windowed mutual matcher with the Hamming
// distances from the tensor cores (tcgen05): the batch path of matcher 0.
//
// FindMatchesInLod (match_features_cpu.cpp:66-150): for every query, the
// features of the other frame's same level and its two neighbours whose
// LOD-0 position lies within +-0.1 W0 in x and +-0.1 H0 in y are the
// candidates; best and second-best Hamming distance; the query is matched iff
// (float)best < 0.85f * (float)second.  The integer matcher (k_match)
// computes exactly the in-window distances.  Here the distances come in tiles
// from the tensor cores, and the window becomes a mask in the epilogue:
//
//   * a work unit is 128 queries that follow each other in the band-grouped
//     query order of one level (one horizontal band, x-consecutive), and its
//     candidates are, per pool level, the range of that band's x-sorted
//     candidate list covering the union of the 128 windows, in tiles of 128
//     list rows (k_win_plan writes the units);
//   * the operands are the descriptors as FP8 rows (bit = 8.0 or 0, so a 0/1
//     dot product times 64) with the popcount / row extension of k_bf_mma,
//     written by k_describe in query order and in list order; nine
//     tcgen05.mma (K = 32) per tile leave in TMEM the exact integer key
//       key = 32 (2 dot - popc(b) + 257) + s,   32 <= key <= 16447,
//     (s = the candidate's list position mod 32), a larger key a smaller
//     distance: distance = popc(a) + 257 - (key >> 5);
//   * the epilogue keeps, per query row, only the columns of its own window:
//     list positions [m0, m1) (the x test, exact through the list's column
//     table as in k_match) and candidate rows y in [ylo, yhi] of the
//     candidate's level (the y test |cy - y s| <= 0.1 H0 in f32, an interval
//     of integer rows found with the reference's own comparison);
//   * best and second best run on 16-bit keys two columns at a time, as in
//     k_bf_mma.  A tie on the best leaves equal distances, which fail the
//     ratio test, so the result does not depend on the scan order: the same
//     lists as k_match, bit for bit.
//
// Every mbarrier wait is bounded; past the limit the kernel records
// USLAM_ERR_TMA_TIMEOUT, drains what it issued (again bounded), frees its TMEM
// and leaves.
#include <cuda_runtime.h>
#include <stdint.h>

#include "uslam_internal.h"

namespace uslam {

struct MatchSegDev {
    int pair;
    int dir;
    int level;
};

// One work unit: 128 query rows of one (pair, direction, level, band) and,
// per pool level k (0: same level, 1: one below, 2: one above), the first
// candidate-list row of its tiles (a multiple of 32) and the tile count.
struct WinUnit {
    int pair, dir, level, band;
    int qrow;   // first operand row of the query tile in the query frame's wq8
    int qpos;   // first query-order position of the tile
    int nq;     // queries in the tile (0: empty slot)
    int pool2;  // the pool (the three levels' features) holds at least 2
    int pl[3];  // pool level of range k (-1: none)
    int c0[3];  // first list row of range k
    int nt[3];  // tiles of range k
    int pad[3];
};
static_assert(sizeof(WinUnit) == 80, "unit record");

namespace {

constexpr int NB = USLAM_MATCH_BANDS;
constexpr int WN_CONSUMERS = 16;                     // 4 lane quarters x 4 column quarters
constexpr int WN_THREADS = 32 * (WN_CONSUMERS + 1);  // plus one producer warp
constexpr int WN_M = 128;                            // queries per unit (TMEM lanes)
constexpr int WN_N = 128;                            // candidate rows per tile
constexpr int WN_STAGES = 3;                         // candidate tiles in flight
constexpr int WN_BUFS = 4;                           // TMEM accumulators (tile t -> t % 4)
constexpr uint32_t WN_ROW = 256;                     // FP8 values per descriptor
constexpr uint32_t WN_A_BYTES = WN_M * WN_ROW;       // 32 KB, double-buffered
constexpr uint32_t WN_AX_BYTES = WN_M * 32;          // query-side extension (constant)
constexpr uint32_t WN_B_BYTES = WN_N * WN_ROW;       // 32 KB
constexpr uint32_t WN_BX_BYTES = WN_N * 32;          // candidate extension rows
constexpr uint32_t WN_Y_BYTES = WN_N * 2;            // candidate y (u16)
constexpr uint32_t WN_SMEM = 2 * WN_A_BYTES + WN_AX_BYTES + WN_STAGES * (WN_B_BYTES + WN_BX_BYTES) +
                             WN_BUFS * WN_Y_BYTES;
constexpr uint32_t WN_TMEM_COLS = 512;
constexpr uint32_t kWaitLimit = 1u << 16;  // try_wait attempts per wait (each suspends up to kWaitHintNs)
constexpr uint32_t kWaitHintNs = 10000u;
// M = N = 128, D f32, A/B E4M3, K-major
constexpr uint32_t kIdesc = (1u << 4) | ((uint32_t)(WN_N >> 3) << 17) | ((uint32_t)(WN_M >> 4) << 24);
constexpr uint32_t kEmpty16 = 0xFFFFFFFFu;  // an x or y range no value matches (both halves 0xFFFF)

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity) {
    const uint32_t a = saddr(b);
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(kWaitHintNs)
            : "memory");
        if (done) return true;
    }
    return false;
}
// 1D bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(b))
                 : "memory");
}
// Shared-memory matrix descriptor, K-major, no swizzle (core matrices of 8
// rows x 16 bytes; LBO = step along K, SBO = step between 8-row groups).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
__device__ __forceinline__ void mma_f8(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(b))
                 : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32_issue(uint32_t addr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(addr)
        : "memory");
}
// Wait for this thread's tcgen05.ld results; the registers pass through the
// statement, so no use of them can be scheduled before the wait.
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                   "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                 :
                 : "memory");
}

__device__ __forceinline__ uint32_t vmax2(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("max.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
__device__ __forceinline__ uint32_t vmin2(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
__device__ __forceinline__ void top2x2(uint32_t& b, uint32_t& s, uint32_t key) {
    s = vmax2(s, vmin2(b, key));
    b = vmax2(b, key);
}
__device__ __forceinline__ void top2x2_merge(uint32_t& b, uint32_t& s, uint32_t b2, uint32_t s2) {
    s = vmax2(vmin2(b, b2), vmax2(s, s2));
    b = vmax2(b, b2);
}
// 16-bit key of a 32-column group at tile column base (0 = none) -> (key >> 5) << 8 | column
__device__ __forceinline__ uint32_t widen(uint32_t k16, uint32_t base) {
    return k16 ? (((k16 >> 5) << 8) | (base + (k16 & 31u))) : 0u;
}
__device__ __forceinline__ void top2_merge(uint32_t& b, uint32_t& s, uint32_t b2, uint32_t s2) {
    s = max(min(b, b2), max(s, s2));
    b = max(b, b2);
}
// The keys of two adjacent accumulator columns, packed as 16-bit halves: each
// key is the integer in the low bits of value + 2^23.
__device__ __forceinline__ uint32_t acc_key2(uint32_t a, uint32_t b) {
    const uint32_t ka = __float_as_uint(__uint_as_float(a) + 8388608.0f);
    const uint32_t kb = __float_as_uint(__uint_as_float(b) + 8388608.0f);
    return __byte_perm(ka, kb, 0x5410);
}
// 0xFFFF in each 16-bit half whose value lies outside [lo, hi] (u16x2): the
// clamp leaves a value unchanged exactly when it is inside, and d * 0xFFFF
// spreads d in {0, 1} per half over the half without carry between halves.
__device__ __forceinline__ uint32_t outside2(uint32_t v, uint32_t lo, uint32_t hi) {
    const uint32_t d = vmin2(vmin2(vmax2(v, lo), hi) ^ v, 0x00010001u);
    return d * 0xFFFFu;
}
__device__ __forceinline__ uint32_t outside2_xy(uint32_t y, uint32_t ylo, uint32_t yhi, uint32_t c, uint32_t clo,
                                                uint32_t chi) {
    const uint32_t e = (vmin2(vmax2(y, ylo), yhi) ^ y) | (vmin2(vmax2(c, clo), chi) ^ c);
    return vmin2(e, 0x00010001u) * 0xFFFFu;
}

// Element k (0, 1, 2) of three values held in registers (no indexed array).
template <typename T>
__device__ __forceinline__ T pick3(int k, T a, T b, T c) {
    return k == 0 ? a : (k == 1 ? b : c);
}

__device__ __forceinline__ float lod_scale(int lod) {
    float s = 1.0f;  // match_features_cpu.cpp:58-64
    for (int i = 0; i < lod; ++i) s = s * 1.2f;
    return s;
}
// First xb in [0, w] with (float)xb * s >= lo (w if none).
__device__ int first_col_ge(float lo, float s, int w) {
    int xb = (int)fminf(fmaxf(floorf(lo / s) - 1.0f, 0.0f), (float)w);
    while (xb > 0 && (float)(xb - 1) * s >= lo) --xb;
    while (xb < w && !((float)xb * s >= lo)) ++xb;
    return xb;
}
// Last xb in [-1, w - 1] with (float)xb * s <= hi (-1 if none).
__device__ int last_col_le(float hi, float s, int w) {
    int xb = (int)fminf(fmaxf(floorf(hi / s) + 1.0f, -1.0f), (float)(w - 1));
    while (xb < w - 1 && (float)(xb + 1) * s <= hi) ++xb;
    while (xb >= 0 && !((float)xb * s <= hi)) --xb;
    return xb;
}
// Rows yb of a level of height h (scale s) that pass the reference's y test
// for a query at LOD-0 y cy: !(|cy - (float)yb * s| > dy) in f32
// (match_features_cpu.cpp:123-126).  (float)yb * s grows with yb, so they
// form an interval [*lo, *hi]; empty -> *lo > *hi.
__device__ void y_rows(float cy, float dy, float s, int h, int* lo, int* hi) {
    auto pass = [&](int yb) { return !(fabsf(cy - (float)yb * s) > dy); };
    int a = (int)fminf(fmaxf(floorf((cy - dy) / s) - 1.0f, 0.0f), (float)(h - 1));
    while (a > 0 && pass(a - 1)) --a;
    while (a < h && !pass(a) && (float)a * s < cy) ++a;
    if (a >= h || !pass(a)) {
        *lo = 1;
        *hi = 0;
        return;
    }
    int e = (int)fminf(fmaxf(floorf((cy + dy) / s) + 1.0f, (float)a), (float)(h - 1));
    while (e > a && !pass(e)) --e;
    while (e + 1 < h && pass(e + 1)) ++e;
    *lo = a;
    *hi = e;
}

}  // namespace

// ------------------------------------------------------------------ plan ----
// The units of one (pair, direction, level) per CTA: for band b, query tile
// t covers query-order positions qband[b] + 128 t .. + 127 of the level; the
// union of their windows spans list positions [c0, c1) of band b's list of
// each pool level (the queries are x-sorted, so the union runs from the first
// query's window start to the last one's end).  Slots past the level's tiles
// are marked empty.
__global__ void __launch_bounds__(64) k_win_plan(const FrameDev* __restrict__ frames,
                                                 const PairDev* __restrict__ pairs,
                                                 const MatchSegDev* __restrict__ segs, int umax,
                                                 WinUnit* __restrict__ units) {
    const MatchSegDev sg = segs[blockIdx.x];
    const PairDev& P = pairs[sg.pair];
    const FrameDev& Q = frames[sg.dir == 0 ? P.curr : P.prev];
    const FrameDev& B = frames[sg.dir == 0 ? P.prev : P.curr];
    const int l = sg.level;
    const uint32_t* qband = Q.colstart[l] + (size_t)NB * (size_t)(Q.w[l] + 1);
    uint32_t nt[NB], tot = 0;
    for (int b = 0; b < NB; ++b) {
        nt[b] = (qband[b + 1] - qband[b] + 127u) / 128u;
        tot += nt[b];
    }
    const int L = B.levels;
    uint32_t pool = B.kept[l];
    if (l > 0) pool += B.kept[l - 1];
    if (l + 1 < L) pool += B.kept[l + 1];
    const float ql = lod_scale(l);
    for (int j = threadIdx.x; j < umax; j += blockDim.x) {
        WinUnit u;
        u.pair = sg.pair;
        u.dir = sg.dir;
        u.level = l;
        u.band = 0;
        u.qrow = 0;
        u.qpos = 0;
        u.nq = 0;
        u.pool2 = pool >= 2u ? 1 : 0;
        u.pad[0] = u.pad[1] = u.pad[2] = 0;
        for (int k = 0; k < 3; ++k) {
            u.pl[k] = -1;
            u.c0[k] = 0;
            u.nt[k] = 0;
        }
        if ((uint32_t)j < tot) {
            uint32_t t = (uint32_t)j, qoff = 0;
            int b = 0;
            while (t >= nt[b]) {
                t -= nt[b];
                qoff += nt[b] * 128u;
                ++b;
            }
            u.band = b;
            u.qpos = (int)(qband[b] + 128u * t);
            u.nq = (int)min(128u, qband[b + 1] - (uint32_t)u.qpos);
            u.qrow = (int)((uint32_t)l * (uint32_t)Q.wq_rows + qoff + 128u * t);
            if (pool >= 2u) {
                const uint32_t* qo = Q.qorder[l];
                const uint32_t* fe = Q.feats[l];
                const float xf = (float)(uint32_t)__uint_as_float(fe[(size_t)qo[u.qpos] * 12u]) * ql;
                const float xl = (float)(uint32_t)__uint_as_float(fe[(size_t)qo[u.qpos + u.nq - 1] * 12u]) * ql;
                const float lo = xf - P.max_dx, hi = xl + P.max_dx;
                for (int k = 0; k < 3; ++k) {
                    const int pl = k == 0 ? l : (k == 1 ? l - 1 : l + 1);
                    if (pl < 0 || pl >= L) continue;
                    const float ps = lod_scale(pl);
                    const int wpl = B.w[pl];
                    const int xlo = first_col_ge(lo, ps, wpl), xhi = last_col_le(hi, ps, wpl);
                    if (xlo > xhi) continue;
                    const uint32_t* col = B.colstart[pl] + (size_t)b * (size_t)(wpl + 1);
                    const uint32_t c0 = col[xlo], c1 = col[xhi + 1];
                    if (c0 >= c1) continue;
                    u.pl[k] = pl;
                    u.c0[k] = (int)(c0 & ~31u);
                    u.nt[k] = (int)((c1 - (c0 & ~31u) + (uint32_t)WN_N - 1u) / (uint32_t)WN_N);
                }
            }
        }
        units[(size_t)blockIdx.x * (size_t)umax + (size_t)j] = u;
    }
}

// ------------------------------------------------------------------ match ---
// Persistent, one CTA per SM.  Units are taken in slot order with a stride
// of the grid; both roles walk the same unit sequence and count the tiles
// they pass (tk, across units): tile tk uses candidate stage tk % 3 and TMEM
// accumulator tk % 4, and the query tile of the u-th unit with tiles uses A
// buffer u % 2.
__global__ void __launch_bounds__(WN_THREADS, 1)
k_win_mma(const FrameDev* __restrict__ frames, const PairDev* __restrict__ pairs, const WinUnit* __restrict__ units,
          int nslots, uint32_t* err) {
    extern __shared__ __align__(1024) uint8_t wn_smem[];
    __shared__ __align__(8) uint64_t a_full[2], a_empty[2], b_full[WN_STAGES], b_empty[WN_STAGES], acc_full[WN_BUFS],
        acc_empty[WN_BUFS], y_full[WN_BUFS];
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail, s_stop;
    __shared__ uint32_t s_mb[4][WN_M], s_ms[4][WN_M];  // per row: the four warps' partial top-2
    __shared__ int32_t s_mi[4][WN_M];
    uint8_t* sA = wn_smem;                                      // 2 query tiles
    uint8_t* sAx = sA + 2 * WN_A_BYTES;                         // query-side extension
    uint8_t* sB = sAx + WN_AX_BYTES;                            // stage s: sB + s * WN_B_BYTES
    uint8_t* sBx = sB + WN_STAGES * WN_B_BYTES;                 // stage s: sBx + s * WN_BX_BYTES
    uint16_t* sY = reinterpret_cast<uint16_t*>(sBx + WN_STAGES * WN_BX_BYTES);  // buffer b: sY + b * WN_N
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    volatile int* fail = &s_fail;

    // query-side extension, the same for every row: 16 x -32 (0xE0), 32 (0x60),
    // 1, 1 (0x38), 32, zeros
    for (int i = t; i < (int)WN_AX_BYTES; i += WN_THREADS) {
        const int r = i >> 5, k = i & 31;
        const uint8_t v = k < 16 ? 0xE0 : (k == 16 || k == 19) ? 0x60 : (k == 17 || k == 18) ? 0x38 : 0x00;
        sAx[(r >> 3) * 256 + (k >> 4) * 128 + (r & 7) * 16 + (k & 15)] = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (t == 0) {
        s_fail = 0;
        s_stop = 0;
        for (int i = 0; i < 2; ++i) {
            bar_init(&a_full[i], 1);
            bar_init(&a_empty[i], 1);
        }
        for (int i = 0; i < WN_STAGES; ++i) {
            bar_init(&b_full[i], 1);
            bar_init(&b_empty[i], 1);
        }
        for (int i = 0; i < WN_BUFS; ++i) {
            bar_init(&acc_full[i], 1);
            bar_init(&acc_empty[i], WN_CONSUMERS);
            bar_init(&y_full[i], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == WN_CONSUMERS) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&s_tmem)),
                     "r"(WN_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;

    if (warp == WN_CONSUMERS) {
        // ------------------------------------------------ producer (one lane)
        if (lane == 0) {
            const uint64_t desc_ax = smem_desc(saddr(sAx), 128u, 256u);
            // a cursor over the tile sequence: unit slot g (with its record),
            // range k, tile i of the range
            struct Cur {
                uint32_t g;
                int k, i;
                WinUnit u;
            };
            auto first_tile = [&](Cur& c) {  // from slot c.g on: the first unit with a tile
                for (; c.g < (uint32_t)nslots; c.g += gridDim.x) {
                    c.u = units[c.g];
                    if (c.u.nq == 0) continue;
                    for (c.k = 0; c.k < 3; ++c.k)
                        if (c.u.nt[c.k] > 0) {
                            c.i = 0;
                            return;
                        }
                }
            };
            // advance by one tile; returns true when the unit changed
            auto advance = [&](Cur& c) -> bool {
                if (++c.i < c.u.nt[c.k]) return false;
                for (++c.k; c.k < 3; ++c.k)
                    if (c.u.nt[c.k] > 0) {
                        c.i = 0;
                        return false;
                    }
                c.g += gridDim.x;
                first_tile(c);
                return true;
            };
            Cur ld{(uint32_t)blockIdx.x, 0, 0, WinUnit{}}, mm{(uint32_t)blockIdx.x, 0, 0, WinUnit{}};
            first_tile(ld);
            first_tile(mm);
            // tiles loaded / given to the MMAs; units whose query tile was
            // loaded / waited for by the MMAs / whose MMAs were all issued
            uint32_t kk_ld = 0, kk_mm = 0, ua_ld = 0, a_iss = 0, a_wt = 0, ua_mm = 0;
            bool ld_new = true, mm_new = true;  // the cursor sits on its unit's first tile
            int64_t last_mma = -1;              // tile index of the last MMA group committed
            bool ok = true;
            while (mm.g < (uint32_t)nslots && ok && !*fail) {
                // loads up to WN_STAGES tiles ahead of the MMAs; a unit's query
                // tile only once the MMAs of the unit two before it (the same A
                // buffer) were all issued, so every wait below is for work
                // already handed to the tensor cores
                while (ok && ld.g < (uint32_t)nslots && kk_ld < kk_mm + WN_STAGES) {
                    if (ld_new && ua_ld > ua_mm + 1u) break;
                    const PairDev& Pl = pairs[ld.u.pair];
                    const FrameDev& Bf = frames[ld.u.dir == 0 ? Pl.prev : Pl.curr];
                    if (ld_new) {
                        const FrameDev& Qf = frames[ld.u.dir == 0 ? Pl.curr : Pl.prev];
                        const uint32_t ab = ua_ld & 1u;
                        ok = bar_wait(&a_empty[ab], ((ua_ld >> 1) + 1u) & 1u);
                        if (!ok) break;
                        bar_expect(&a_full[ab], WN_A_BYTES);
                        bulk_load(sA + ab * WN_A_BYTES, Qf.wq8 + (size_t)(ld.u.qrow >> 3) * 2048u, WN_A_BYTES,
                                  &a_full[ab]);
                        a_iss = ua_ld + 1u;
                        ld_new = false;
                    }
                    const uint32_t st = kk_ld % WN_STAGES;
                    ok = bar_wait(&b_empty[st], ((kk_ld / WN_STAGES) + 1u) & 1u);
                    if (!ok) break;
                    const uint32_t row = (uint32_t)(NB * ld.u.pl[ld.k] + ld.u.band) * (uint32_t)Bf.wc_rows +
                                         (uint32_t)ld.u.c0[ld.k] + (uint32_t)ld.i * WN_N;
                    bar_expect(&b_full[st], WN_B_BYTES + WN_BX_BYTES);
                    bulk_load(sB + st * WN_B_BYTES, Bf.wc8 + (size_t)(row >> 3) * 2048u, WN_B_BYTES, &b_full[st]);
                    bulk_load(sBx + st * WN_BX_BYTES, Bf.wcext + (size_t)(row >> 3) * 256u, WN_BX_BYTES, &b_full[st]);
                    ++kk_ld;
                    if (advance(ld)) {
                        ++ua_ld;
                        ld_new = true;
                    }
                }
                if (!ok) break;
                // MMAs of tile kk_mm
                const PairDev& Pm = pairs[mm.u.pair];
                const FrameDev& Bm = frames[mm.u.dir == 0 ? Pm.prev : Pm.curr];
                const uint32_t ab = ua_mm & 1u;
                if (mm_new) {
                    ok = bar_wait(&a_full[ab], (ua_mm >> 1) & 1u);
                    a_wt = ua_mm + 1u;
                }
                const uint32_t st = kk_mm % WN_STAGES, buf = kk_mm % WN_BUFS, use = kk_mm / WN_BUFS;
                ok = ok && bar_wait(&b_full[st], (kk_mm / WN_STAGES) & 1u) && bar_wait(&acc_empty[buf], (use + 1u) & 1u);
                if (!ok) break;
                // the candidates' y of this tile, for the consumers of accumulator buf
                const uint32_t row = (uint32_t)(NB * mm.u.pl[mm.k] + mm.u.band) * (uint32_t)Bm.wc_rows +
                                     (uint32_t)mm.u.c0[mm.k] + (uint32_t)mm.i * WN_N;
                bar_expect(&y_full[buf], WN_Y_BYTES);
                bulk_load(sY + buf * WN_N, Bm.wcy + row, WN_Y_BYTES, &y_full[buf]);
                fence_after();
                const uint64_t da = smem_desc(saddr(sA + ab * WN_A_BYTES), 128u, 2048u);
                const uint64_t db = smem_desc(saddr(sB + st * WN_B_BYTES), 128u, 2048u);
                const uint64_t dbx = smem_desc(saddr(sBx + st * WN_BX_BYTES), 128u, 256u);
                const uint32_t d = tmem + buf * (uint32_t)WN_N;
#pragma unroll
                for (int k = 0; k < 8; ++k) mma_f8(d, da + (uint64_t)(16 * k), db + (uint64_t)(16 * k), k > 0);
                mma_f8(d, desc_ax, dbx, 1u);
                mma_commit(&acc_full[buf]);
                mma_commit(&b_empty[st]);
                last_mma = (int64_t)kk_mm;
                ++kk_mm;
                mm_new = advance(mm);
                if (mm_new) {
                    mma_commit(&a_empty[ab]);  // the unit's query tile is read once its MMAs complete
                    ++ua_mm;
                }
            }
            if (!ok) *fail = 1;
            if (*fail) {
                atomicOr(err, USLAM_ERR_TMA_TIMEOUT);
                // drain what was issued, each wait bounded: the last MMA group
                // and its y copy, the candidate tiles loaded after it, the query
                // tiles loaded but not yet waited for
                if (last_mma >= 0) {
                    const uint32_t b = (uint32_t)(last_mma % WN_BUFS), par = (uint32_t)((last_mma / WN_BUFS) & 1);
                    bar_wait(&acc_full[b], par);
                    bar_wait(&y_full[b], par);
                }
                for (int64_t i = max(last_mma + 1, (int64_t)kk_ld - WN_STAGES); i < (int64_t)kk_ld; ++i)
                    bar_wait(&b_full[i % WN_STAGES], (uint32_t)((i / WN_STAGES) & 1));
                for (uint32_t u = a_wt; u < a_iss; ++u) bar_wait(&a_full[u & 1u], (u >> 1) & 1u);
            }
        }
        __syncwarp();
    } else {
        // ----------------------------------------------------------- consumers
        // warp w: TMEM lane quarter w % 4 (query rows), column quarter w / 4
        // (32 columns) of every tile
        const int q4 = warp & 3, cq = warp >> 2;
        const int row = 32 * q4 + lane;
        const int slot = cq;
        uint32_t kk = 0;
        for (uint32_t g = blockIdx.x; g < (uint32_t)nslots; g += gridDim.x) {
            const WinUnit u = units[g];
            if (u.nq == 0) continue;
            const PairDev& P = pairs[u.pair];
            const FrameDev& Q = frames[u.dir == 0 ? P.curr : P.prev];
            const FrameDev& B = frames[u.dir == 0 ? P.prev : P.curr];
            const int l = u.level;
            const bool valid = row < u.nq;
            // this row's query and its window per pool level: list positions
            // [m0, m1) and candidate rows [ylo, yhi], as u16x2 pairs
            uint32_t qi = 0, pq = 0;
            uint32_t xlo2[3], xhi2[3], ylo2[3], yhi2[3];
            int m0[3], m1[3];
            {
                float cx = 0.0f, cy = 0.0f;
                if (valid) {
                    qi = __ldg(Q.qorder[l] + u.qpos + row);
                    const uint32_t* rec = Q.feats[l] + (size_t)qi * 12u;
                    const float ql = lod_scale(l);
                    cx = (float)(uint32_t)__uint_as_float(rec[0]) * ql;
                    cy = (float)(uint32_t)__uint_as_float(rec[1]) * ql;
                    const uint4 d0 = *reinterpret_cast<const uint4*>(rec + 4);
                    const uint4 d1 = *reinterpret_cast<const uint4*>(rec + 8);
                    pq = (uint32_t)(__popc(d0.x) + __popc(d0.y) + __popc(d0.z) + __popc(d0.w) + __popc(d1.x) +
                                    __popc(d1.y) + __popc(d1.z) + __popc(d1.w));
                }
                const float lo = cx - P.max_dx, hi = cx + P.max_dx;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    xlo2[k] = xhi2[k] = ylo2[k] = yhi2[k] = kEmpty16;
                    m0[k] = 1;
                    m1[k] = 0;
                    const int pl = u.pl[k];
                    if (!valid || pl < 0 || u.nt[k] == 0) continue;
                    const float ps = lod_scale(pl);
                    const int wpl = B.w[pl];
                    const int xlo = first_col_ge(lo, ps, wpl), xhi = last_col_le(hi, ps, wpl);
                    if (xlo > xhi) continue;
                    const uint32_t* col = B.colstart[pl] + (size_t)u.band * (size_t)(wpl + 1);
                    const int a = (int)__ldg(col + xlo), e = (int)__ldg(col + xhi + 1);
                    int ya, yb;
                    y_rows(cy, P.max_dy, ps, B.h[pl], &ya, &yb);
                    if (a >= e || ya > yb) continue;
                    m0[k] = a;
                    m1[k] = e;
                    xlo2[k] = (uint32_t)a * 0x00010001u;
                    xhi2[k] = (uint32_t)(e - 1) * 0x00010001u;
                    ylo2[k] = (uint32_t)ya * 0x00010001u;
                    yhi2[k] = (uint32_t)yb * 0x00010001u;
                }
            }
            uint32_t best = 0u, second = 0u;  // widened keys; 0 = no candidate
            int32_t bidx = -1;
            bool bad = false;
            const int nt0 = u.nt[0], nt1 = u.nt[1], nt2 = u.nt[2];
            const int NT = nt0 + nt1 + nt2;
            for (int n = 0; n < NT; ++n) {
                const uint32_t tk = kk + (uint32_t)n;
                // range k of tile n and its tile i within the range
                const int k = n < nt0 ? 0 : (n < nt0 + nt1 ? 1 : 2);
                const int i = n - (k == 0 ? 0 : (k == 1 ? nt0 : nt0 + nt1));
                const uint32_t buf = tk % WN_BUFS, use = tk / WN_BUFS;
                bad = bad || *fail != 0 || !bar_wait(&acc_full[buf], use & 1u) || !bar_wait(&y_full[buf], use & 1u);
                fence_after();
                // tcgen05.ld is warp-wide: a warp reads the accumulator only if
                // every lane saw it complete
                const bool go = __all_sync(0xffffffffu, !bad);
                uint32_t r[32];
                uint32_t yw = 0u;  // lane j < 16: the y of this warp's columns 2 j, 2 j + 1
                if (go) {
                    const uint32_t addr = tmem + ((uint32_t)(32 * q4) << 16) + buf * (uint32_t)WN_N + (uint32_t)(32 * cq);
                    tmem_ld32_issue(addr, r);
                    yw = reinterpret_cast<const uint32_t*>(sY + buf * WN_N + 32 * cq)[lane & 15];
                    tmem_wait(r);
                }
                // the accumulator and its y are read: release them to the producer
                fence_before();
                __syncwarp();
                if (lane == 0) bar_arrive(&acc_empty[buf]);
                if (!go) {
                    bad = true;
                    continue;
                }
                // this range's window of the row, and the list position of this
                // warp's first column
                const int c0k = pick3(k, u.c0[0], u.c0[1], u.c0[2]);
                const int plk = pick3(k, u.pl[0], u.pl[1], u.pl[2]);
                const int M0 = pick3(k, m0[0], m0[1], m0[2]), M1 = pick3(k, m1[0], m1[1], m1[2]);
                const uint32_t YL = pick3(k, ylo2[0], ylo2[1], ylo2[2]), YH = pick3(k, yhi2[0], yhi2[1], yhi2[2]);
                const int cb = c0k + i * WN_N + 32 * cq;
                uint32_t cbk[4] = {0u, 0u, 0u, 0u}, csk[4] = {0u, 0u, 0u, 0u};
                // every column of the group inside this row's x range?
                const bool inside = M0 <= cb && cb + 32 <= M1;
                if (__all_sync(0xffffffffu, inside)) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const uint32_t y2 = __shfl_sync(0xffffffffu, yw, j);
                        const uint32_t key = acc_key2(r[2 * j], r[2 * j + 1]) & ~outside2(y2, YL, YH);
                        top2x2(cbk[j & 3], csk[j & 3], key);
                    }
                } else {
                    const uint32_t XL = pick3(k, xlo2[0], xlo2[1], xlo2[2]), XH = pick3(k, xhi2[0], xhi2[1], xhi2[2]);
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const uint32_t y2 = __shfl_sync(0xffffffffu, yw, j);
                        const uint32_t c2 = (uint32_t)(cb + 2 * j) | ((uint32_t)(cb + 2 * j + 1) << 16);
                        const uint32_t key = acc_key2(r[2 * j], r[2 * j + 1]) & ~outside2_xy(y2, YL, YH, c2, XL, XH);
                        top2x2(cbk[j & 3], csk[j & 3], key);
                    }
                }
                top2x2_merge(cbk[0], csk[0], cbk[1], csk[1]);
                top2x2_merge(cbk[2], csk[2], cbk[3], csk[3]);
                top2x2_merge(cbk[0], csk[0], cbk[2], csk[2]);
                // tile column of the group's first column: 32 cq
                const uint32_t gb = (uint32_t)(32 * cq);
                uint32_t tb = widen(cbk[0] & 0xffffu, gb), ts = widen(csk[0] & 0xffffu, gb);
                top2_merge(tb, ts, widen(cbk[0] >> 16, gb), widen(csk[0] >> 16, gb));
                if (tb > best) {
                    const uint32_t lrow = (uint32_t)(NB * plk + u.band) * (uint32_t)B.wc_rows +
                                          (uint32_t)(c0k + i * WN_N) + (tb & 255u);
                    bidx = __ldg(B.wcid + lrow);
                }
                top2_merge(best, second, tb, ts);
            }
            kk += (uint32_t)NT;
            if (bad) *fail = 1;
            // merge the four warps of each query row (named barrier 1: the
            // consumer warps only)
            s_mb[slot][row] = best;
            s_ms[slot][row] = second;
            s_mi[slot][row] = bidx;
            asm volatile("bar.sync 1, %0;" ::"r"(32 * WN_CONSUMERS) : "memory");
            if (slot == 0) {
                for (int o = 1; o < 4; ++o) {
                    const uint32_t ob = s_mb[o][row];
                    if (ob > best) bidx = s_mi[o][row];
                    top2_merge(best, second, ob, s_ms[o][row]);
                }
                if (valid && !*fail) {
                    // distance = popc(a) + 257 - (key >> 5), key >> 5 = widened key >> 8
                    const uint32_t db = best == 0u ? 0xffffffu : pq + 257u - (best >> 8);
                    const uint32_t ds = second == 0u ? 0xffffffu : pq + 257u - (second >> 8);
                    const int32_t res = (u.pool2 && bidx >= 0 && (float)db < 0.85f * (float)ds) ? bidx : -1;
                    const int capq = Q.cap;
                    if (u.dir == 0) P.b2a[(size_t)l * capq + qi] = res;
                    else P.a2b[(size_t)l * capq + qi] = res;
                }
                if (warp == 0 && lane == 0) s_stop = *fail;
            }
            asm volatile("bar.sync 1, %0;" ::"r"(32 * WN_CONSUMERS) : "memory");  // s_m*, s_stop
            if (s_stop) break;
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == WN_CONSUMERS)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(WN_TMEM_COLS) : "memory");
}

// ---------------------------------------------------------------- launch ----

cudaError_t set_win_mma_smem() {
    return cudaFuncSetAttribute(k_win_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WN_SMEM);
}

// Unit slots per (pair, direction, level) for levels of at most `cap` features.
int win_units_per_seg(int cap) { return (cap + WN_M - 1) / WN_M + NB; }

cudaError_t launch_win_match(const FrameDev* frames, const PairDev* pairs, const void* msegs, int nmsegs, int umax,
                             void* units, int num_sms, uint32_t* err, cudaStream_t st) {
    if (nmsegs <= 0) return cudaSuccess;
    auto* U = static_cast<WinUnit*>(units);
    k_win_plan<<<nmsegs, 64, 0, st>>>(frames, pairs, static_cast<const MatchSegDev*>(msegs), umax, U);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int nslots = nmsegs * umax;
    k_win_mma<<<min(num_sms, nslots), WN_THREADS, WN_SMEM, st>>>(frames, pairs, U, nslots, err);
    return cudaGetLastError();
}

size_t win_unit_bytes() { return sizeof(WinUnit); }

}  // namespace uslam
