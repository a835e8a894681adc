// bf_tc.cu — brute-force top-2 Hamming matching on the tensor cores (tcgen05).
//
// The brute-force matcher (matcher 2; the same result as k_bruteforce,
// matcher 1) compares every feature of frame prev with every feature of frame
// curr.  With each descriptor bit as an FP8 E4M3 value (0x38 = 1.0, 0x00 =
// 0.0), popc(a & b) is the dot product of two 256-element 0/1 vectors, and
//   Hamming(a, b) = popc(a) + popc(b) - 2 popc(a & b).
// Every partial sum of such a dot product is an integer <= 256, exact in the
// f32 accumulator whatever the summation order, so the distances are exact.
//
// k_describe writes each frame's descriptors in that form, with each bit as
// 8.0 (uslam_internal.h: bf8 rows of 256 bytes in the K-major no-swizzle
// core-matrix layout), and a 32-value extension row per feature: its
// popcount split into 16 integers <= 16, 256, its row index within its
// 32-row group (s) split into two integers <= 16, 1.  Against the constant
// query-side extension (16 x -32, 32, 1, 1, 32) a ninth K step adds
// -32 popc(b) + 32 * 257 + s, so the accumulator holds the integer
//   key = 32 (2 dot - popc(b) + 257) + s,   32 <= key <= 16447,
// every product and partial sum exact in f32.  For a query a larger key is a
// smaller distance (distance = popc(a) + 257 - (key >> 5)), and s tells the
// columns of a 32-column group apart.
//
// One persistent CTA per SM holds 512 TMEM columns: two buffers of two
// 128 x 128 f32 accumulators.  A work unit is 256 queries of one pair (one
// accumulator per 128) against the pair's train set, or a share of it when
// the train set is split.  A producer warp stages the query tile (64 KB) and
// the train tiles (128 rows: 32 KB + 4 KB extension, four stages) by bulk
// copies and issues, per train tile, nine tcgen05.mma (K = 32) into each
// accumulator of one buffer; sixteen consumer warps (four per TMEM lane
// quarter: accumulator x 64-column group) read the other buffer with
// tcgen05.ld, release it, and reduce it, one query row per thread.  The keys
// fit 16 bits: adding 2^23 in f32 leaves a key in the low bits of the sum, a
// byte permute packs columns j and j + 32 of a 64-column group into one
// register, and the top-2 runs on both halves at once with max/min.u16x2 over
// four independent chains.  At the end of a group the 16-bit keys widen to
// (key >> 5) << 8 | column-in-tile.  A tie on the best leaves equal
// distances, which fail the ratio test (the rule of k_bruteforce), so the
// result does not depend on the scan order.  At most 1024 pairs per launch.
//
// Every mbarrier wait is bounded (attempts that suspend the warp until the
// phase completes or a hint expires, so waiting warps leave the issue slots
// to the others); past the limit the kernel records
// USLAM_ERR_TMA_TIMEOUT, drains what it issued (again bounded), frees its TMEM
// and leaves.
#include <cuda_runtime.h>
#include <stdint.h>

#include "uslam_internal.h"

namespace uslam {

namespace {

constexpr int TC_CONSUMERS = 16;                // epilogue warps: 4 per TMEM lane quarter (2 accumulators x 2 column halves)
constexpr int TC_THREADS = 32 * (TC_CONSUMERS + 1);    // plus one producer warp
constexpr int TC_M = 128;                       // queries per accumulator (TMEM lanes)
constexpr int TC_Q = 2 * TC_M;                  // queries per work unit: two accumulators share each train tile
constexpr int TC_N = 128;                       // train rows per tile
constexpr int TC_STAGES = 4;                    // train tiles in flight
constexpr uint32_t TC_ROW_BYTES = 256;          // 256 FP8 values per descriptor
constexpr uint32_t TC_A_BYTES = TC_Q * TC_ROW_BYTES;   // 64 KB
constexpr uint32_t TC_AX_BYTES = TC_M * 32;            // query-side extension (constant)
constexpr uint32_t TC_B_BYTES = TC_N * TC_ROW_BYTES;   // 32 KB
constexpr uint32_t TC_BX_BYTES = TC_N * 32;            // train-side extension rows
constexpr uint32_t TC_SMEM = TC_A_BYTES + TC_AX_BYTES + TC_STAGES * (TC_B_BYTES + TC_BX_BYTES);
constexpr uint32_t TC_TMEM_COLS = 512;          // 2 buffers x 2 accumulators x 128 columns
constexpr uint32_t kWaitLimit = 1u << 16;       // try_wait attempts per wait (each suspends up to kWaitHintNs)
constexpr uint32_t kWaitHintNs = 10000u;        // suspend-time hint of one attempt (the attempt returns at completion)
constexpr int kMaxPairs = 1024;                 // pairs per launch (the unit table lives in shared memory)

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
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity, uint32_t limit = kWaitLimit) {
    const uint32_t a = saddr(b);
    for (uint32_t i = 0; i < limit; ++i) {
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

// Shared-memory matrix descriptor, K-major, no swizzle: core matrices of
// 8 rows x 16 bytes (128 contiguous bytes); LBO = byte step between core
// matrices along K, SBO = byte step between 8-row groups; bits 46-47 = 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f8f6f4: D f32 (bits 4-5 = 1), A and B E4M3
// (0), both K-major, N >> 3 at bit 17, M >> 4 at bit 24 (M = N = 128).
constexpr uint32_t kIdesc = (1u << 4) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

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

// Issue 32 consecutive f32 columns of this thread's TMEM lane (complete after tmem_wait).
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

// Two 16-bit lanes at once: unsigned max / min per halfword.
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
// 16-bit key of group column base + j (0 = none) -> (key >> 5) << 8 | column
__device__ __forceinline__ uint32_t widen(uint32_t k16, uint32_t base) {
    return k16 ? (((k16 >> 5) << 8) | (base + (k16 & 31u))) : 0u;
}
// Key of an accumulator value: the integer in the low bits of value + 2^23.
__device__ __forceinline__ uint32_t acc_key(uint32_t bits) {
    return __float_as_uint(__uint_as_float(bits) + 8388608.0f);
}
// Top-2 of keys (largest first): (b, s) <- the two largest of {b, s, b2, s2}.
__device__ __forceinline__ void top2_merge(uint32_t& b, uint32_t& s, uint32_t b2, uint32_t s2) {
    s = max(min(b, b2), max(s, s2));
    b = max(b, b2);
}

__device__ __forceinline__ uint32_t total_kept(const FrameDev& F) {
    uint32_t n = 0;
    for (int l = 0; l < F.levels; ++l) n += F.kept[l];
    return n;
}

}  // namespace

// Work units: 256 queries of one pair (two 128-row accumulators) against
// the pair's train set, or a share of it when the train set is split.  Both
// roles walk the same unit sequence and count the train tiles they pass
// (kk, across units): tile kk uses stage kk % 3 and accumulator buffer
// kk % 2, and the parity of the barrier phase it waits for follows from kk.
struct TcUnit {
    const PairDev* P;
    const FrameDev* A;
    const FrameDev* B;
    uint32_t nq, nt, qbase, tb, split, nsplit;
    int NT;
};

__device__ __forceinline__ TcUnit tc_unit(const FrameDev* frames, const PairDev* pairs, const SegDev* psegs,
                                          const uint32_t* pref, int npairs, uint32_t g) {
    int lo = 0, hi = npairs - 1;  // pair with pref[p] <= g < pref[p + 1]
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pref[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    TcUnit u;
    u.P = &pairs[psegs[lo].frame];
    u.A = &frames[u.P->prev];
    u.B = &frames[u.P->curr];
    u.nsplit = (uint32_t)max(u.P->bf_splits, 1);
    const uint32_t unit = g - pref[lo];
    const uint32_t qt = unit / u.nsplit;
    u.split = unit - qt * u.nsplit;
    u.qbase = qt * (uint32_t)TC_Q;
    u.nq = total_kept(*u.A);
    u.nt = total_kept(*u.B);
    const uint32_t ntiles = (u.nt + TC_N - 1) / TC_N;
    u.tb = u.split * ntiles / u.nsplit;
    u.NT = (int)((u.split + 1u) * ntiles / u.nsplit - u.tb);
    return u;
}

// Result per query a in a2b (packed (level, index) of its match in curr, or
// -1), or, when the pair's train set is split, one partial record per split
// ((distance << 8) of best and second, best id) merged by the emit kernel.
__global__ void __launch_bounds__(TC_THREADS, 1)
k_bf_mma(const FrameDev* __restrict__ frames, const PairDev* __restrict__ pairs, const SegDev* __restrict__ psegs,
         int npairs, float ratio, uint32_t* err) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    __shared__ __align__(8) uint64_t bar_a, b_full[TC_STAGES], b_empty[TC_STAGES], acc_full[2], acc_empty[2];
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;
    __shared__ uint32_t s_pref[kMaxPairs + 1];
    __shared__ uint32_t s_hb[TC_Q], s_hs[TC_Q];  // second column group's top-2 per query row
    __shared__ int32_t s_hi[TC_Q];
    uint8_t* sA = tc_smem;
    uint8_t* sAx = sA + TC_A_BYTES;
    uint8_t* sB = sAx + TC_AX_BYTES;                   // stage s: sB + s * TC_B_BYTES
    uint8_t* sBx = sB + TC_STAGES * TC_B_BYTES;        // stage s: sBx + s * TC_BX_BYTES
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    volatile int* fail = &s_fail;

    // work units per pair: query blocks x train splits
    for (int p = t; p < npairs; p += TC_THREADS) {
        const PairDev& P = pairs[psegs[p].frame];
        const uint32_t nq = total_kept(frames[P.prev]);
        s_pref[p + 1] = (nq + TC_Q - 1) / TC_Q * (uint32_t)max(P.bf_splits, 1);
    }
    // query-side extension, the same for every row: 16 x -32 (0xE0), 32 (0x60),
    // 1, 1 (0x38), 32, zeros
    for (int i = t; i < (int)TC_AX_BYTES; i += TC_THREADS) {
        const int r = i >> 5, k = i & 31;
        const uint8_t v = k < 16 ? 0xE0 : (k == 16 || k == 19) ? 0x60 : (k == 17 || k == 18) ? 0x38 : 0x00;
        sAx[(r >> 3) * 256 + (k >> 4) * 128 + (r & 7) * 16 + (k & 15)] = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (t == 0) {
        s_fail = 0;
        bar_init(&bar_a, 1);
        for (int i = 0; i < TC_STAGES; ++i) {
            bar_init(&b_full[i], 1);
            bar_init(&b_empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            bar_init(&acc_full[i], 1);
            bar_init(&acc_empty[i], TC_CONSUMERS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == TC_CONSUMERS) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&s_tmem)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    if (t == 0) {
        s_pref[0] = 0;
        for (int p = 0; p < npairs; ++p) s_pref[p + 1] += s_pref[p];
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t total = s_pref[npairs];

    if (warp == TC_CONSUMERS) {
        // ------------------------------------------------ producer (one lane)
        if (lane == 0) {
            // operand descriptors of stage 0 / query tile 0 (K-major, no swizzle)
            const uint64_t desc_a = smem_desc(saddr(sA), 128u, 2048u);
            const uint64_t desc_ax = smem_desc(saddr(sAx), 128u, 256u);
            const uint64_t desc_b = smem_desc(saddr(sB), 128u, 2048u);
            const uint64_t desc_bx = smem_desc(saddr(sBx), 128u, 256u);
            uint32_t kk = 0, units_loaded = 0;
            bool a_pending = false;  // a query tile in flight whose wait gave up
            int64_t last_mma = -1;  // tile index of the last MMA group committed
            int64_t loaded_to = 0;  // tiles [.., loaded_to) have had their loads issued
            auto load_b = [&](const TcUnit& u, uint32_t tile_kk, uint32_t n) -> bool {
                const uint32_t st = tile_kk % TC_STAGES;
                // the stage's previous tile (tile_kk - 3) must have been read by its MMAs
                if (!bar_wait(&b_empty[st], ((tile_kk / TC_STAGES) + 1u) & 1u)) return false;
                bar_expect(&b_full[st], TC_B_BYTES + TC_BX_BYTES);
                const uint32_t tile = u.tb + n;
                bulk_load(sB + st * TC_B_BYTES, u.B->bf8 + (size_t)tile * TC_B_BYTES, TC_B_BYTES, &b_full[st]);
                bulk_load(sBx + st * TC_BX_BYTES, u.B->bfext + (size_t)tile * TC_BX_BYTES, TC_BX_BYTES, &b_full[st]);
                loaded_to = (int64_t)tile_kk + 1;
                return true;
            };
            for (uint32_t g = blockIdx.x; g < total && !*fail; g += gridDim.x) {
                const TcUnit u = tc_unit(frames, pairs, psegs, s_pref, npairs, g);
                if (u.NT <= 0) continue;
                bool ok = true;
                // the query tiles are rewritten: the previous unit's MMAs must be done
                if (last_mma >= 0) ok = bar_wait(&acc_full[last_mma & 1], (uint32_t)(last_mma >> 1) & 1u);
                if (ok) {
                    bar_expect(&bar_a, TC_A_BYTES);
                    bulk_load(sA, u.A->bf8 + (size_t)u.qbase * TC_ROW_BYTES, TC_A_BYTES, &bar_a);
                    // the launch's first query-tile wait may be shortened (a test hook)
                    const int fw = u.A->match_first_wait;
                    ok = bar_wait(&bar_a, units_loaded & 1u, units_loaded == 0 && fw >= 0 ? (uint32_t)fw : kWaitLimit);
                    a_pending = !ok;
                    ++units_loaded;
                }
                for (int n = 0; n < TC_STAGES - 1 && n < u.NT && ok; ++n) ok = load_b(u, kk + (uint32_t)n, (uint32_t)n);
                for (int n = 0; n < u.NT && ok; ++n) {
                    const uint32_t tk = kk + (uint32_t)n, st = tk % TC_STAGES, buf = tk & 1u;
                    ok = bar_wait(&b_full[st], (tk / TC_STAGES) & 1u) &&
                         bar_wait(&acc_empty[buf], ((tk >> 1) + 1u) & 1u);
                    if (!ok) break;
                    fence_after();
                    // descriptor start addresses advance in 16-byte units
                    const uint64_t db = desc_b + (uint64_t)((st * TC_B_BYTES) >> 4);
                    const uint64_t dbx = desc_bx + (uint64_t)((st * TC_BX_BYTES) >> 4);
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const uint64_t da = desc_a + (uint64_t)((h * (TC_A_BYTES / 2)) >> 4);
                        const uint32_t d = tmem + buf * (uint32_t)(2 * TC_N) + (uint32_t)(h * TC_N);
#pragma unroll
                        for (int k = 0; k < 8; ++k) mma_f8(d, da + (uint64_t)(16 * k), db + (uint64_t)(16 * k), k > 0);
                        mma_f8(d, desc_ax, dbx, 1u);
                    }
                    mma_commit(&acc_full[buf]);
                    mma_commit(&b_empty[st]);
                    last_mma = (int64_t)tk;
                    // the stage of tile tk - 1 takes tile tk + TC_STAGES - 1
                    if (n + TC_STAGES - 1 < u.NT)
                        ok = load_b(u, tk + (uint32_t)(TC_STAGES - 1), (uint32_t)(n + TC_STAGES - 1));
                }
                kk += (uint32_t)u.NT;
                if (!ok) *fail = 1;
            }
            if (*fail) {
                atomicOr(err, USLAM_ERR_TMA_TIMEOUT);
                // drain what was issued, each wait bounded
                if (last_mma >= 0) bar_wait(&acc_full[last_mma & 1], (uint32_t)(last_mma >> 1) & 1u);
                for (int64_t i = max(last_mma + 1, loaded_to - TC_STAGES); i < loaded_to; ++i)
                    bar_wait(&b_full[i % TC_STAGES], (uint32_t)(i / TC_STAGES) & 1u);
                // the query tile whose wait gave up lands before the CTA leaves
                if (a_pending) bar_wait(&bar_a, (units_loaded - 1u) & 1u);
            }
        }
        __syncwarp();
    } else {
        // ----------------------------------------------------------- consumers
        // warp w: TMEM lane quarter w % 4, accumulator (query tile) (w / 4) % 2,
        // columns 64 (w / 8) .. + 63 of each train tile
        const int quarter = warp & 3, half = (warp >> 2) & 1, cgrp = warp >> 3;
        const int row = 32 * quarter + lane;
        const uint32_t s0 = (uint32_t)(64 * cgrp);  // this warp's first column in a tile
        uint32_t kk = 0;
        for (uint32_t g = blockIdx.x; g < total; g += gridDim.x) {
            const TcUnit u = tc_unit(frames, pairs, psegs, s_pref, npairs, g);
            uint32_t best = 0u, second = 0u;  // widened keys; 0 = no candidate
            int32_t bidx = -1;
            bool bad = false;
            for (int n = 0; n < u.NT; ++n) {
                const uint32_t tk = kk + (uint32_t)n, buf = tk & 1u;
                bad = bad || *fail != 0 || !bar_wait(&acc_full[buf], (tk >> 1) & 1u);
                fence_after();
                // tcgen05.ld is warp-wide: a warp reads the accumulator only if
                // every lane saw it complete
                const bool go = __all_sync(0xffffffffu, !bad);
                uint32_t r0[32], r1[32];
                if (go) {
                    const uint32_t col = buf * (uint32_t)(2 * TC_N) + (uint32_t)(half * TC_N) + s0;
                    const uint32_t addr = tmem + ((uint32_t)(32 * quarter) << 16) + col;
                    tmem_ld32_issue(addr, r0);
                    tmem_ld32_issue(addr + 32u, r1);
                    tmem_wait(r0);
                    tmem_wait(r1);
                }
                // the accumulator is read: release it to the producer
                fence_before();
                __syncwarp();
                if (lane == 0) bar_arrive(&acc_empty[buf]);
                if (go) {
                    const uint32_t base = (u.tb + (uint32_t)n) * (uint32_t)TC_N;
                    const uint32_t valid = u.nt - base < (uint32_t)TC_N ? u.nt - base : (uint32_t)TC_N;
                    uint32_t cb[4] = {0u, 0u, 0u, 0u}, cs[4] = {0u, 0u, 0u, 0u};
                    if (valid == (uint32_t)TC_N) {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            top2x2(cb[j & 3], cs[j & 3], __byte_perm(acc_key(r0[j]), acc_key(r1[j]), 0x5410));
                    } else {  // the last tile of the train set: columns past its end are no candidates
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            const uint32_t k0 = s0 + (uint32_t)j, k1 = k0 + 32u;
                            const uint32_t lo = k0 < valid ? (acc_key(r0[j]) & 0xffffu) : 0u;
                            const uint32_t hi = k1 < valid ? (acc_key(r1[j]) << 16) : 0u;
                            top2x2(cb[j & 3], cs[j & 3], lo | hi);
                        }
                    }
                    top2x2_merge(cb[0], cs[0], cb[1], cs[1]);
                    top2x2_merge(cb[2], cs[2], cb[3], cs[3]);
                    top2x2_merge(cb[0], cs[0], cb[2], cs[2]);
                    uint32_t tb = widen(cb[0] & 0xffffu, s0), ts = widen(cs[0] & 0xffffu, s0);
                    top2_merge(tb, ts, widen(cb[0] >> 16, s0 + 32u), widen(cs[0] >> 16, s0 + 32u));
                    if (tb > best) bidx = __ldg(u.B->bfid + base + (tb & 255u));
                    top2_merge(best, second, tb, ts);
                } else {
                    bad = true;
                }
            }
            kk += (uint32_t)max(u.NT, 0);
            if (bad) *fail = 1;
            // merge the two column groups of each query row (named barrier 1:
            // the consumer warps only)
            const int slot_row = half * TC_M + row;
            if (cgrp == 1) {
                s_hb[slot_row] = best;
                s_hs[slot_row] = second;
                s_hi[slot_row] = bidx;
            }
            asm volatile("bar.sync 1, %0;" ::"r"(32 * TC_CONSUMERS) : "memory");
            const uint32_t q = u.qbase + (uint32_t)slot_row;
            if (cgrp == 0 && !bad && q < u.nq) {
                const uint32_t ob = s_hb[slot_row];
                if (ob > best) bidx = s_hi[slot_row];
                top2_merge(best, second, ob, s_hs[slot_row]);
                const FrameDev& A = *u.A;
                const int32_t qid = __ldg(A.bfid + q);
                const size_t slot = (size_t)USLAM_PACK_LEVEL(qid) * A.cap + (size_t)USLAM_PACK_INDEX(qid);
                // distance = popc(a) + 257 - (key >> 5), key >> 5 = widened key >> 8
                const uint32_t pq = __ldg(A.bfpop + q);
                const uint32_t db = best == 0u ? 0xffffffu : pq + 257u - (best >> 8);
                const uint32_t ds = second == 0u ? 0xffffffu : pq + 257u - (second >> 8);
                if (u.nsplit == 1u) {
                    u.P->a2b[slot] = (u.nt >= 2u && bidx >= 0 && (float)db < ratio * (float)ds) ? bidx : -1;
                } else {
                    const size_t stride = (size_t)A.levels * A.cap;
                    *reinterpret_cast<uint4*>(u.P->bf_part + (u.split * stride + slot) * 4u) =
                        make_uint4(db << 8, ds << 8, (uint32_t)bidx, 0u);
                }
            }
            asm volatile("bar.sync 1, %0;" ::"r"(32 * TC_CONSUMERS) : "memory");  // s_h* reused by the next unit
            if (*fail) break;
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == TC_CONSUMERS)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

// The kernel's dynamic shared memory limit, per device: called when a batch
// for the tensor-core matcher is created, with its device current.
cudaError_t set_bf_mma_smem() {
    return cudaFuncSetAttribute(k_bf_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
}

cudaError_t launch_bf_mma(const FrameDev* frames, const PairDev* pairs, const SegDev* psegs, int npairs, float ratio,
                          int grid, uint32_t* err, cudaStream_t st) {
    if (npairs <= 0) return cudaSuccess;
    if (npairs > kMaxPairs) return cudaErrorInvalidValue;
    k_bf_mma<<<grid, TC_THREADS, TC_SMEM, st>>>(frames, pairs, psegs, npairs, ratio, err);
    return cudaGetLastError();
}

}  // namespace uslam
