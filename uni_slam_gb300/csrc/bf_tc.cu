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
// k_describe writes each frame's descriptors in that form (uslam_internal.h:
// bf8 rows of 256 bytes in the K-major no-swizzle core-matrix layout, and a
// 32-value extension row per feature: its popcount split into 16 integers
// <= 16, then 16 x 16.0).  Against a constant query-side extension (16 x -0.5,
// 16 x 1.0) a ninth K step adds -popc(b) / 2 + 256, so the accumulator holds
//   v = dot - popc(b) / 2 + 256 = 512 - (distance - popc(a)) / 2,
// a half-integer in [128, 384]: every product and partial sum is exact.
// For a query, a larger v is a smaller distance.
//
// One persistent CTA per SM holds 512 TMEM columns: two 128 x 256 f32
// accumulators.  A work unit is 128 queries of one pair against its train set
// (or a share of it when the pair's train set is split): the query tile
// (32 KB) and the train tiles (64 KB + 8 KB extension, double-buffered) are
// staged by bulk copies; one thread issues nine tcgen05.mma (K = 32 each) per
// train tile into one accumulator while eight warps reduce the other (two
// warps per TMEM lane quarter, 128 columns each; tcgen05.ld, one query row per
// thread) to keys and a branch-free top-2 over four independent chains.
//
// Key of a candidate: bits(v) | slot.  v is positive with its low 8 mantissa
// bits zero, so keys order like v; max/min on keys keep the two largest v
// (the two smallest distances); a tie on the best leaves equal distances,
// which fail the ratio test (the rule of k_bruteforce), so the result does
// not depend on the scan order.
//
// Every mbarrier wait is bounded; past the limit the kernel records
// USLAM_ERR_TMA_TIMEOUT, drains what it issued (again bounded), frees its TMEM
// and leaves.
#include <cuda_runtime.h>
#include <stdint.h>

#include "uslam_internal.h"

namespace uslam {

namespace {

constexpr int TC_THREADS = 256;                 // 8 warps: two per TMEM lane quarter
constexpr int TC_M = 128;                       // queries per work unit
constexpr int TC_N = 256;                       // train rows per tile
constexpr uint32_t TC_ROW_BYTES = 256;          // 256 FP8 values per descriptor
constexpr uint32_t TC_A_BYTES = TC_M * TC_ROW_BYTES;   // 32 KB
constexpr uint32_t TC_B_BYTES = TC_N * TC_ROW_BYTES;   // 64 KB
constexpr uint32_t TC_AX_BYTES = TC_M * 32;            // query-side extension (constant)
constexpr uint32_t TC_BX_BYTES = TC_N * 32;            // train-side extension rows
constexpr uint32_t TC_SMEM = TC_A_BYTES + TC_AX_BYTES + 2 * (TC_B_BYTES + TC_BX_BYTES);
constexpr uint32_t TC_TMEM_COLS = 512;          // two accumulators of TC_N columns
constexpr uint32_t kWaitLimit = 1u << 24;       // try_wait polls per wait
constexpr int kMaxPairs = 4096;

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n) : "memory");
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
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
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
// (0), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
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
__device__ __forceinline__ void tmem_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Top-2 of keys (largest first): (b, s) <- the two largest of {b, s, key}.
__device__ __forceinline__ void top2(uint32_t& b, uint32_t& s, uint32_t key) {
    s = max(s, min(b, key));
    b = max(b, key);
}
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

// Result per query a in a2b (packed (level, index) of its match in curr, or
// -1), or, when the pair's train set is split, one partial record per split
// ((distance << 8) of best and second, best id) merged by the emit kernel.
__global__ void __launch_bounds__(TC_THREADS, 1)
k_bf_mma(const FrameDev* __restrict__ frames, const PairDev* __restrict__ pairs, const SegDev* __restrict__ psegs,
         int npairs, float ratio, uint32_t* err) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    __shared__ __align__(8) uint64_t bar_a, bar_b[2], bar_m[2];
    __shared__ uint32_t s_tmem;
    __shared__ uint32_t s_pref[kMaxPairs + 1];
    __shared__ uint32_t s_hb[TC_M], s_hs[TC_M];  // the second column half's top-2 per query row
    __shared__ int32_t s_hi[TC_M];
    uint8_t* sA = tc_smem;
    uint8_t* sAx = sA + TC_A_BYTES;
    uint8_t* sB[2] = {sAx + TC_AX_BYTES, sAx + TC_AX_BYTES + TC_B_BYTES};
    uint8_t* sBx[2] = {sAx + TC_AX_BYTES + 2 * TC_B_BYTES, sAx + TC_AX_BYTES + 2 * TC_B_BYTES + TC_BX_BYTES};
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int quarter = warp & 3, half = warp >> 2;
    const int row = 32 * quarter + lane;  // this thread's query row (TMEM lane)

    // work units per pair: query tiles x train splits
    for (int p = t; p < npairs; p += TC_THREADS) {
        const PairDev& P = pairs[psegs[p].frame];
        const uint32_t nq = total_kept(frames[P.prev]);
        s_pref[p + 1] = (nq + TC_M - 1) / TC_M * (uint32_t)max(P.bf_splits, 1);
    }
    // query-side extension, the same for every row: 16 x -0.5 (0xB0), 16 x 1.0 (0x38)
    for (int i = t; i < (int)TC_AX_BYTES; i += TC_THREADS) {
        const int r = i >> 5, k = i & 31;
        sAx[(r >> 3) * 256 + (k >> 4) * 128 + (r & 7) * 16 + (k & 15)] = k < 16 ? 0xB0 : 0x38;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (t == 0) {
        bar_init(&bar_a, 1);
        bar_init(&bar_b[0], 1);
        bar_init(&bar_b[1], 1);
        bar_init(&bar_m[0], 1);
        bar_init(&bar_m[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
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

    // parities of the next completion to wait for (bar_a / bar_b: thread 0
    // only; bar_m: every thread, uniformly)
    uint32_t ph_a = 0, ph_b0 = 0, ph_b1 = 0, ph_m0 = 0, ph_m1 = 0;
    uint32_t pend_b = 0, pend_m = 0;  // thread 0: copies / MMA groups issued and not yet waited for
    bool fail = false;

    // thread 0: stage train tile `tile` of B into buffer s
    auto load_b = [&](const FrameDev& B, uint32_t tile, int s) {
        bar_expect(&bar_b[s], TC_B_BYTES + TC_BX_BYTES);
        bulk_load(sB[s], B.bf8 + (size_t)tile * TC_B_BYTES, TC_B_BYTES, &bar_b[s]);
        bulk_load(sBx[s], B.bfext + (size_t)tile * TC_BX_BYTES, TC_BX_BYTES, &bar_b[s]);
        pend_b |= 1u << s;
    };
    // thread 0: the nine MMAs of the train tile in buffer s into accumulator s
    auto issue_mma = [&](int s) {
        fence_after();
        const uint32_t a0 = saddr(sA), b0 = saddr(sB[s]), d = tmem + (uint32_t)(s * TC_N);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            mma_f8(d, smem_desc(a0 + 256u * k, 128u, 2048u), smem_desc(b0 + 256u * k, 128u, 2048u), k > 0);
        mma_f8(d, smem_desc(saddr(sAx), 128u, 256u), smem_desc(saddr(sBx[s]), 128u, 256u), 1u);
        mma_commit(&bar_m[s]);
        pend_m |= 1u << s;
    };

    for (uint32_t g = blockIdx.x; g < total && !fail; g += gridDim.x) {
        int lo = 0, hi = npairs - 1;  // pair with s_pref[p] <= g < s_pref[p + 1]
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_pref[mid] <= g) lo = mid;
            else hi = mid - 1;
        }
        const PairDev& P = pairs[psegs[lo].frame];
        const FrameDev& A = frames[P.prev];
        const FrameDev& B = frames[P.curr];
        const uint32_t nsplit = (uint32_t)max(P.bf_splits, 1);
        const uint32_t unit = g - s_pref[lo];
        const uint32_t qt = unit / nsplit, split = unit - qt * nsplit;
        const uint32_t nq = total_kept(A), nt = total_kept(B);
        const uint32_t ntiles = (nt + TC_N - 1) / TC_N;
        const uint32_t tb = split * ntiles / nsplit, te = (split + 1u) * ntiles / nsplit;
        const int NT = (int)(te - tb);
        uint32_t best = 0u, second = 0u;  // keys; 0 = no candidate
        int32_t bidx = -1;

        if (NT > 0) {
            if (t == 0) {
                bar_expect(&bar_a, TC_A_BYTES);
                bulk_load(sA, A.bf8 + (size_t)qt * TC_A_BYTES, TC_A_BYTES, &bar_a);
                load_b(B, tb, 0);
                if (NT > 1) load_b(B, tb + 1u, 1);
                bool ok = bar_wait(&bar_a, ph_a);
                ph_a ^= 1u;
                ok = ok && bar_wait(&bar_b[0], ph_b0);
                ph_b0 ^= 1u;
                pend_b &= ~1u;
                if (ok) issue_mma(0);
                else fail = true;
            }
            fail = __syncthreads_or(fail);
            for (int n = 0; n < NT && !fail; ++n) {
                const int b = n & 1;
                if (t == 0 && n + 1 < NT) {
                    // the next tile's MMAs into the other accumulator (read out
                    // before the last barrier)
                    const int nb = b ^ 1;
                    const bool ok = bar_wait(&bar_b[nb], nb ? ph_b1 : ph_b0);
                    if (nb) ph_b1 ^= 1u;
                    else ph_b0 ^= 1u;
                    pend_b &= ~(1u << nb);
                    if (ok) issue_mma(nb);
                    else fail = true;
                }
                // this tile's accumulator
                const bool landed = bar_wait(&bar_m[b], b ? ph_m1 : ph_m0);
                if (b) ph_m1 ^= 1u;
                else ph_m0 ^= 1u;
                if (t == 0) pend_m &= ~(1u << b);
                if (!landed) fail = true;
                fence_after();
                if (t == 0 && !fail && n + 2 < NT) load_b(B, tb + (uint32_t)n + 2u, b);  // its buffer is free
                // tcgen05.ld is warp-wide: a warp reads the accumulator only if
                // every lane saw it complete
                if (__all_sync(0xffffffffu, !fail)) {
                    const uint32_t base = (tb + (uint32_t)n) * (uint32_t)TC_N;
                    const uint32_t valid = nt - base < (uint32_t)TC_N ? nt - base : (uint32_t)TC_N;
                    uint32_t cb[4] = {0u, 0u, 0u, 0u}, cs[4] = {0u, 0u, 0u, 0u};
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        uint32_t r0[32], r1[32];
                        const uint32_t col = (uint32_t)(b * TC_N + half * 128 + 64 * c);
                        const uint32_t addr = tmem + ((uint32_t)(32 * quarter) << 16) + col;
                        tmem_ld32_issue(addr, r0);
                        tmem_ld32_issue(addr + 32u, r1);
                        tmem_wait();
                        const uint32_t s0 = (uint32_t)(half * 128 + 64 * c);
                        if (valid == (uint32_t)TC_N) {
#pragma unroll
                            for (int j = 0; j < 32; ++j) {
                                top2(cb[j & 3], cs[j & 3], r0[j] | (s0 + (uint32_t)j));
                                top2(cb[j & 3], cs[j & 3], r1[j] | (s0 + 32u + (uint32_t)j));
                            }
                        } else {  // the last tile of the train set: columns past its end are no candidates
#pragma unroll
                            for (int j = 0; j < 32; ++j) {
                                const uint32_t k0 = s0 + (uint32_t)j, k1 = k0 + 32u;
                                top2(cb[j & 3], cs[j & 3], k0 < valid ? (r0[j] | k0) : 0u);
                                top2(cb[j & 3], cs[j & 3], k1 < valid ? (r1[j] | k1) : 0u);
                            }
                        }
                    }
                    top2_merge(cb[0], cs[0], cb[1], cs[1]);
                    top2_merge(cb[2], cs[2], cb[3], cs[3]);
                    top2_merge(cb[0], cs[0], cb[2], cs[2]);
                    if (cb[0] > best) bidx = __ldg(B.bfid + base + (cb[0] & 255u));
                    top2_merge(best, second, cb[0], cs[0]);
                }
                fence_before();
                fail = __syncthreads_or(fail);
            }
        }
        // merge the two column halves of each query row
        if (half == 1) {
            s_hb[row] = best;
            s_hs[row] = second;
            s_hi[row] = bidx;
        }
        __syncthreads();
        const uint32_t q = qt * TC_M + (uint32_t)row;
        if (half == 0 && !fail && q < nq) {
            const uint32_t ob = s_hb[row];
            if (ob > best) bidx = s_hi[row];
            top2_merge(best, second, ob, s_hs[row]);
            const int32_t qid = __ldg(A.bfid + q);
            const size_t slot = (size_t)USLAM_PACK_LEVEL(qid) * A.cap + (size_t)USLAM_PACK_INDEX(qid);
            // distance = popc(a) + 512 - 2 v
            const uint32_t pq = __ldg(A.bfpop + q);
            const uint32_t db = best == 0u ? 0xffffffu : pq + 512u - (uint32_t)(2.0f * __uint_as_float(best & ~255u));
            const uint32_t ds =
                second == 0u ? 0xffffffu : pq + 512u - (uint32_t)(2.0f * __uint_as_float(second & ~255u));
            if (nsplit == 1u) {
                P.a2b[slot] = (nt >= 2u && bidx >= 0 && (float)db < ratio * (float)ds) ? bidx : -1;
            } else {
                const size_t stride = (size_t)A.levels * A.cap;
                *reinterpret_cast<uint4*>(P.bf_part + (split * stride + slot) * 4u) =
                    make_uint4(db << 8, ds << 8, (uint32_t)bidx, 0u);
            }
        }
        __syncthreads();  // s_hb / s_hs / s_hi are rewritten by the next unit
    }
    if (fail && t == 0) {
        atomicOr(err, USLAM_ERR_TMA_TIMEOUT);
        // drain what this thread issued, each wait bounded
        if (pend_b & 1u) bar_wait(&bar_b[0], ph_b0);
        if (pend_b & 2u) bar_wait(&bar_b[1], ph_b1);
        if (pend_m & 1u) bar_wait(&bar_m[0], ph_m0);
        if (pend_m & 2u) bar_wait(&bar_m[1], ph_m1);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

cudaError_t launch_bf_mma(const FrameDev* frames, const PairDev* pairs, const SegDev* psegs, int npairs, float ratio,
                          int grid, uint32_t* err, cudaStream_t st) {
    if (npairs <= 0) return cudaSuccess;
    if (npairs > kMaxPairs) return cudaErrorInvalidValue;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(k_bf_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_bf_mma<<<grid, TC_THREADS, TC_SMEM, st>>>(frames, pairs, psegs, npairs, ratio, err);
    return cudaGetLastError();
}

}  // namespace uslam
