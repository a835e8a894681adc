// kernels.cu — sm_103a kernels of the GB300 feature front-end.
//
//   k_pyramid       every pyramid level as f32 rows of 16-byte pitch (level 0 =
//                   u8 / 255, levels >= 1 one bilinear tap of LOD0): the
//                   source of k_detect's tile loads
//   k_detect   (K1) TMA-staged level tile + halo, FAST response + cull, blur
//                   cache (or, in the cfg profile, FAST 9-of-16 at 20/255 +
//                   3x3 NMS)
//   k_blur_border   blur cache beyond the level edges (BRIEF points outside)
//   k_band_count, k_band_write
//                   ordered keypoint compaction over 32-row bands, cap
//   k_xsort         the matcher's lists: per horizontal band an x-sorted
//                   candidate list, and the band-grouped query order
//   k_describe (K2) orientation (one lane per keypoint of a warp's group) +
//                   256-bit rotated BRIEF (the warp's lanes take 8 tests each)
//   k_bacc_init     empties the b -> a accumulators before each k_match
//   k_match_rank, k_match_order
//                   k_match's claim order: query groups by estimated cost
//   k_match    (K3) windowed top-2 Hamming search of both directions, one
//                   distance per pair; a warp claims groups of 32 x-adjacent
//                   queries of the previous set in one band
//   k_mutual        mutual cross-check (b's search read from its accumulator)
//                   and ordered match output
//   k_bruteforce    brute-force top-2 matching (no window, no cross-check) on
//                   the integer pipes; the tensor-core form is k_bf_mma
//                   (bf_tc.cu)
//
// Arithmetic contract: binary32, round-to-nearest-even, no FMA contraction
// (the library is compiled with --fmad=false), evaluation order as in the
// reference shaders.  Every kernel is bit-exact against the CPU oracle.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/uslam_canon.h"
#include "uslam_internal.h"

namespace uslam {

// K1 tile geometry: TW x TH output pixels (a template parameter pair, one of
// kTileShapes), halo HX columns / HY rows (HY_CFG with the cfg profile, whose
// 3x3 NMS needs the FAST score one pixel beyond the tile).
constexpr int HX = USLAM_TILE_HX;
constexpr int HY = USLAM_TILE_HY;
constexpr int HY_CFG = USLAM_TILE_HY_CFG;
constexpr int K1_THREADS = 256;
// Spin limit of a tile load's mbarrier wait (try_wait polls); past it the
// kernel records USLAM_ERR_TMA_TIMEOUT and leaves the tile.
constexpr uint32_t kTmaWaitLimit = 1u << 20;
// cfg detection profile threshold: 20 grey levels on the u8/255 scale.
constexpr float kCfgThreshold = 20.0f / 255.0f;

// Matcher band of a LOD-0 y in a frame of height H (rows [b H / B, (b + 1) H / B)).
__device__ __forceinline__ int match_band(float y, float H) {
    const int b = (int)floorf(y * (float)USLAM_MATCH_BANDS / H);
    return b < 0 ? 0 : (b >= USLAM_MATCH_BANDS ? USLAM_MATCH_BANDS - 1 : b);
}

// Bresenham circle of radius 3 (resources/detect_corners.wgsl:31-32) as
// compile-time constants: in the unrolled loops the shared-memory offsets fold
// into immediates.
__device__ __forceinline__ constexpr int circle_x(int i) {
    return i == 0 ? 0 : i == 1 ? 1 : i == 2 ? 2 : i <= 5 ? 3 : i == 6 ? 2 : i == 7 ? 1 : i == 8 ? 0
         : i == 9 ? -1 : i == 10 ? -2 : i <= 13 ? -3 : i == 14 ? -2 : -1;
}
// A quarter turn maps point i to point i + 4 ((x, y) -> (-y, x)), so y_i = -x_(i+4).
__device__ __forceinline__ constexpr int circle_y(int i) { return -circle_x((i + 4) & 15); }

// Tint robustness clamp of textureLoad coordinates: min(u32(c), n - 1).
__device__ __forceinline__ int tint_clamp(int c, int n) {
    const unsigned u = (unsigned)c;
    return u < (unsigned)n ? (int)u : n - 1;
}

// Clamp-to-edge index of an integer-valued float (may be huge or negative).
__device__ __forceinline__ int edge_index(float f, int n) {
    if (f <= 0.0f) return 0;
    if (f >= (float)(n - 1)) return n - 1;
    return (int)f;
}

// FAST response at smem cell (r, c): 1 + longest non-wrapping run of
// |centre - p_i| > 0.15, kept iff > 9 (detect_corners.wgsl:58-81).
template <int SW>
__device__ __forceinline__ uint32_t fast_response(const float (*sm)[SW], int r, int c) {
    const float center = sm[r][c];
    // every non-wrapping run of >= 9 of the 16 points contains points 7 and 8
    if (!(fabsf(center - sm[r + 3][c + 1]) > 0.15f && fabsf(center - sm[r + 3][c]) > 0.15f)) return 0u;
    uint32_t m = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const float p = sm[r + circle_y(i)][c + circle_x(i)];
        m |= (fabsf(center - p) > 0.15f ? 1u : 0u) << i;
    }
    // run >= 9 test: AND of the mask shifted by 0..8
    uint32_t t = m & (m >> 1);
    t &= t >> 2;
    t &= t >> 4;
    t &= t >> 1;
    if (t == 0u) return 0u;
    uint32_t run = 0;
    while (m) {
        m &= m << 1;
        ++run;
    }
    return run + 1u;
}

// Longest run of ones of a 16-bit circle mask, wrapping around (16 if all set).
__device__ __forceinline__ uint32_t circular_run(uint32_t m) {
    if (m == 0xffffu) return 16u;
    uint32_t x = m | (m << 16), run = 0;
    while (x) {
        x &= x << 1;
        ++run;
    }
    return run;
}

// cfg profile corner test at smem cell (r, c): FAST 9-of-16 with wrap-around,
// brighter iff p - c > T, darker iff c - p > T (T = 20/255).  Returns the
// score (sum over i = 0..15 of (|p_i - c| - T) for the points of the
// qualifying polarity, added in index order) and the arc length (longest
// circular run, 9..16) in *arc; 0 and 0 if not a corner.
template <int SW>
__device__ __forceinline__ float cfg_corner(const float (*sm)[SW], int r, int c, uint32_t* arc) {
    const float center = sm[r][c];
    float d[16];
    uint32_t mb = 0, md = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const float p = sm[r + circle_y(i)][c + circle_x(i)];
        d[i] = p - center;
        mb |= (d[i] > kCfgThreshold ? 1u : 0u) << i;
        md |= ((center - p) > kCfgThreshold ? 1u : 0u) << i;
    }
    *arc = 0u;
    if (__popc(mb) < 9 && __popc(md) < 9) return 0.0f;
    const uint32_t rb = circular_run(mb), rd = circular_run(md);
    if (rb < 9u && rd < 9u) return 0.0f;
    const bool bright = rb >= 9u;
    const uint32_t m = bright ? mb : md;
    float score = 0.0f;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        if (!((m >> i) & 1u)) continue;
        const float dv = bright ? d[i] : (sm[r][c] - sm[r + circle_y(i)][c + circle_x(i)]);
        score = score + (dv - kCfgThreshold);
    }
    *arc = bright ? rb : rd;
    return score;
}

// Packed binary32 products (sm_100 family mul.f32x2): one instruction rounds
// each lane to nearest even exactly as the scalar mul.rn would, so two
// independent products cost one issue slot with unchanged bits.  Sums stay
// scalar: ptxas (CUDA 13.0) contracts mul.rn.f32x2 feeding add.rn.f32x2 into
// one fused multiply-add (a single rounding) in spite of .rn and
// --fmad=false, while a packed product feeding a scalar add.rn is kept as two
// roundings.
__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

// Left-to-right sum of four packed products, lane by lane, in scalar adds.
__device__ __forceinline__ float2 sum4(float2 p, float2 q, float2 r, float2 t) {
    float x = p.x, y = p.y;
    x = x + q.x;
    y = y + q.y;
    x = x + r.x;
    y = y + r.y;
    x = x + t.x;
    y = y + t.y;
    return make_float2(x, y);
}

__device__ __forceinline__ bool mask_bit(const uint32_t* mask, int p) {
    return (__ldg(mask + (p >> 5)) >> (p & 31)) & 1u;
}

// ------------------------------------------------------ TMA + mbarrier ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// Bounded wait for phase `parity` of the barrier: true when it completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t i = 0; i < limit; ++i) {
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
// 2D tiled TMA load of the map's box at element coordinates (x, y) into
// shared memory, completing on the barrier (x * 4 bytes is 32-byte aligned
// for every caller: x = tile origin - 8, tile widths multiples of 32).
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// ----------------------------------------------------------- pyramid ----
// Level l of one TW x TH tile into lvl[l] (row pitch lvl_pitch): l = 0 is
// f32(u8) / 255 (provider_base.cpp:121-124), read 8 pixels per 8-byte load
// and stored as two 16-byte vectors; l >= 1 is one canonical bilinear tap of
// LOD0 at the texel centre (create_pyramid.wgsl:11-12).  Sampling
// coordinates depend only on the row or only on the column, so they are
// computed once per tile row / column (the per-pixel operations, so the same
// bits).  The weights (na nb, a nb) and (na b, a b) are packed products and
// the sum is scalar in the written order.
template <int TW, int TH>
__global__ void __launch_bounds__(K1_THREADS)
k_pyramid(const FrameDev* __restrict__ frames, const TileItem* __restrict__ tiles) {
    static_assert(K1_THREADS % TW == 0 && TW % 8 == 0, "tile shape");
    __shared__ float s_lut[256];  // f32(u8) / 255
    __shared__ int2 s_fx[TW];     // LOD0 source columns (x0, x1) per tile column
    __shared__ float2 s_fa[TW];   // (1 - a, a)
    __shared__ int2 s_fy[TH];     // LOD0 source rows (y0, y1) per tile row
    __shared__ float2 s_fnb[TH], s_fb[TH];  // (1 - b, 1 - b), (b, b)
    const TileItem it = tiles[blockIdx.x];
    const FrameDev& F = frames[it.frame];
    const int l = it.level;
    const int w = F.w[l], h = F.h[l];
    const int X0 = it.tx * TW, Y0 = it.ty * TH;
    const int t = threadIdx.x;
    float* const out = F.lvl[l];
    const int lp = F.lvl_pitch[l];
    const uint8_t* img = F.img;
    const int pitch = F.img_pitch;
    s_lut[t] = (float)t / 255.0f;
    if (l == 0) {
        // 8 pixels per thread (8-byte loads): a 64-wide tile of 32 rows is
        // 256 segments, one per thread.  16-byte loads left half the threads
        // without a segment and measured slower (0.151 against 0.144 ms on 64
        // frames of 752x480).
        __syncthreads();
        constexpr int SEGS = TW / 8;
        for (int u = t; u < SEGS * TH; u += K1_THREADS) {
            const int r = u / SEGS;
            const int x = X0 + (u - r * SEGS) * 8, y = Y0 + r;
            if (y >= h || x >= w) continue;
            // x is a multiple of 8 below w, so x + 8 <= the 16-byte image pitch
            const uint2 q = *reinterpret_cast<const uint2*>(img + (size_t)y * pitch + x);
            float v[8];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                v[k] = s_lut[(q.x >> (8 * k)) & 255u];
                v[4 + k] = s_lut[(q.y >> (8 * k)) & 255u];
            }
            float* o = out + (size_t)y * lp + x;
            if (x + 8 <= lp) {
                reinterpret_cast<float4*>(o)[0] = make_float4(v[0], v[1], v[2], v[3]);
                reinterpret_cast<float4*>(o)[1] = make_float4(v[4], v[5], v[6], v[7]);
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (x + k < w) o[k] = v[k];
            }
        }
        return;
    }
    for (int i = t; i < TW + TH; i += K1_THREADS) {
        if (i < TW) {
            const int gx = min(X0 + i, w - 1);
            const float u = (((float)gx + 0.5f) / (float)w) * (float)F.W0 - 0.5f;
            const float fi = floorf(u);
            const float a = u - fi;
            s_fa[i] = make_float2(1.0f - a, a);
            s_fx[i] = make_int2(edge_index(fi, F.W0), edge_index(fi + 1.0f, F.W0));
        } else {
            const int r = i - TW;
            const int gy = min(Y0 + r, h - 1);
            const float v = (((float)gy + 0.5f) / (float)h) * (float)F.H0 - 0.5f;
            const float fj = floorf(v);
            const float b = v - fj, nb = 1.0f - b;
            s_fb[r] = make_float2(b, b);
            s_fnb[r] = make_float2(nb, nb);
            s_fy[r] = make_int2(edge_index(fj, F.H0), edge_index(fj + 1.0f, F.H0));
        }
    }
    __syncthreads();
    const int tx = t % TW;
    const int x = X0 + tx;
    if (x >= w) return;
    const float2 nab = s_fa[tx];
    const int2 fx = s_fx[tx];
    for (int ty = t / TW; ty < TH; ty += K1_THREADS / TW) {
        const int y = Y0 + ty;
        if (y >= h) break;
        const int2 fy = s_fy[ty];
        const uint8_t* r0 = img + (size_t)fy.x * pitch;
        const uint8_t* r1 = img + (size_t)fy.y * pitch;
        const float2 t0 = make_float2(s_lut[__ldg(r0 + fx.x)], s_lut[__ldg(r0 + fx.y)]);
        const float2 t1 = make_float2(s_lut[__ldg(r1 + fx.x)], s_lut[__ldg(r1 + fx.y)]);
        const float2 p0 = mul2_rn(mul2_rn(nab, s_fnb[ty]), t0);
        const float2 p1 = mul2_rn(mul2_rn(nab, s_fb[ty]), t1);
        float val = p0.x;
        val = val + p0.y;
        val = val + p1.x;
        val = val + p1.y;
        out[(size_t)y * lp + x] = val;
    }
}

// ---------------------------------------------------------------- K1 ----
// One TW x TH tile of one level: one TMA load stages the level pixels plus
// halo (written by k_pyramid) in shared memory, then per pixel the FAST
// response, the cull decision and the blur-cache value G(x, y).  The blur
// taps' sampling coordinates depend only on the row or only on the column,
// so they are computed once per tile row / column (same operations as the
// per-pixel formula, hence the same bits).
// Six CTAs per SM (40 registers, no spills): 0.700 against 0.718 ms at five
// (48 registers) and 0.712 at four on the 64-frame step; seven spill.  The
// cfg profile's form spills at 40 and keeps five.
template <int TW, int TH, bool CFG>
__global__ void __launch_bounds__(K1_THREADS, CFG ? 5 : 6)
k_detect(const FrameDev* __restrict__ frames, const TileItem* __restrict__ tiles, int shape, uint32_t* err) {
    constexpr int HY = CFG ? HY_CFG : uslam::HY;
    constexpr int SW = TW + 2 * HX;                   // staged columns [X0 - HX, X0 + TW + HX)
    constexpr int SH = TH + 2 * HY;                   // staged rows [Y0 - HY, Y0 + TH + HY)
    constexpr int BW = TW + 2 * USLAM_TILE_XPAD;      // TMA box columns [X0 - XPAD, X0 + TW + XPAD)
    constexpr int CX = USLAM_TILE_XPAD - HX;          // box column of staged column 0
    static_assert(K1_THREADS % TW == 0 && CX >= 0 && (BW * 4) % 16 == 0 && BW <= 256 && SH <= 256, "tile shape");
    __shared__ __align__(128) float sbox[SH][BW];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_by0[3][TH], s_by1[3][TH];   // blur taps: staged rows per output row
    // blur taps, y weights per output row as pairs: rows j = 0, 1 side by
    // side, and row j = 2 twice
    __shared__ float2 s_b01[TH], s_nb01[TH], s_b22[TH], s_nb22[TH];
    __shared__ float s_score[CFG ? TH + 2 : 1][CFG ? TW + 2 : 1];  // cfg: FAST score, tile + 1 ring
    __shared__ uint8_t s_arc[CFG ? TH + 2 : 1][CFG ? TW + 2 : 1];
    __shared__ uint8_t s_rowfast[TH];  // row taps at fixed offsets (no edge clamp)
    const TileItem it = tiles[blockIdx.x];
    const FrameDev& F = frames[it.frame];
    const int l = it.level;
    const int w = F.w[l], h = F.h[l];
    const int X0 = it.tx * TW, Y0 = it.ty * TH;
    const int t = threadIdx.x;
    const float tex_x = 1.0f / (float)w;
    const float tex_y = 1.0f / (float)h;
    const float off[3] = {-1.2f, 0.0f, 1.2f};

    // 0. one thread starts the tile load; the others build the tap tables
    //    meanwhile.  Box cells outside the level arrive as 0 and are
    //    replaced below.
    if (t == 0) {
        const void* tmap = static_cast<const char*>(F.tmaps) +
                           (size_t)(l * USLAM_TMAPS_PER_LEVEL + shape) * USLAM_TMAP_BYTES;
        mbar_init(&s_bar, 1u);
        mbar_expect_tx(&s_bar, (uint32_t)(SH * BW * 4));
        tma_load_2d(&sbox[0][0], tmap, X0 - USLAM_TILE_XPAD, Y0 - HY, &s_bar);
    }
    for (int i = t; i < TH; i += K1_THREADS) s_rowfast[i] = 1;
    __syncthreads();
    for (int i = t; i < 3 * TH; i += K1_THREADS) {
        // generate_features.wgsl:153-169, y part of the 9 taps
        const int ty = i / 3, k = i % 3;
        const float uvy = ((float)(Y0 + ty) + 0.5f) * tex_y;
        const float offk = k == 0 ? -1.2f : (k == 1 ? 0.0f : 1.2f);
        const float v = (uvy + offk * tex_y) * (float)h - 0.5f;
        const float fj = floorf(v);
        int r0 = edge_index(fj, h) - (Y0 - HY), r1 = edge_index(fj + 1.0f, h) - (Y0 - HY);
        if (Y0 + ty < h && (r0 < 0 || r1 >= SH)) atomicOr(err, USLAM_ERR_SMEM_RANGE);
        const float b = v - fj, nb = 1.0f - b;
        if (k == 2) {
            s_b22[ty] = make_float2(b, b);
            s_nb22[ty] = make_float2(nb, nb);
        } else {
            reinterpret_cast<float*>(&s_b01[ty])[k] = b;
            reinterpret_cast<float*>(&s_nb01[ty])[k] = nb;
        }
        s_by0[k][ty] = min(max(r0, 0), SH - 1);
        s_by1[k][ty] = min(max(r1, 0), SH - 1);
        // the row taps of an interior row sit at rows -2, -1 | d, d + 1 | 1, 2
        // around the pixel (d = -1 or 0): no edge clamp
        const int rr = ty + HY, e = k == 0 ? -2 : (k == 1 ? r0 - rr : 1);
        const bool ok = r1 == r0 + 1 && r0 == rr + e && (k != 1 || e == -1 || e == 0);
        if (!ok) s_rowfast[ty] = 0;
    }
    __syncthreads();  // the barrier is initialised before anyone polls it
    const uint32_t first_limit = F.detect_first_wait < 0 ? kTmaWaitLimit : (uint32_t)F.detect_first_wait;
    const bool landed = mbar_wait(&s_bar, 0u, first_limit);
    if (__syncthreads_or(!landed)) {
        if (t == 0) atomicOr(err, USLAM_ERR_TMA_TIMEOUT);
        mbar_wait(&s_bar, 0u, kTmaWaitLimit);  // the copy in flight lands before the tile is left (full limit)
        return;
    }

    // 1. halo cells outside the level follow the Tint clamp min(u32(c), n - 1)
    //    (a negative coordinate reads the far edge)
    //    Only those cells are visited: whole rows above and below the level,
    //    then the columns left and right of it in the rows between.
    if (X0 < HX || X0 + TW + HX > w || Y0 < HY || Y0 + TH + HY > h) {
        const float* lv = F.lvl[l];
        const int lp = F.lvl_pitch[l];
        const int top = min(max(HY - Y0, 0), SH), bot = min(max(Y0 - HY + SH - h, 0), SH - top);
        const int left = min(max(HX - X0, 0), SW), right = min(max(X0 - HX + SW - w, 0), SW - left);
        const int nrow = (top + bot) * SW, nside = (SH - top - bot) * (left + right);
        for (int idx = t; idx < nrow + nside; idx += K1_THREADS) {
            int r, c;
            if (idx < nrow) {
                const int k = idx / SW;
                r = k < top ? k : SH - bot + (k - top);
                c = idx - k * SW;
            } else {
                const int k = idx - nrow, rr = k / (left + right), cc = k - rr * (left + right);
                r = top + rr;
                c = cc < left ? cc : SW - right + (cc - left);
            }
            const int gy = Y0 - HY + r, gx = X0 - HX + c;
            sbox[r][c + CX] = __ldg(lv + (size_t)tint_clamp(gy, h) * lp + tint_clamp(gx, w));
        }
        __syncthreads();
    }
    // staged cell (r, c) = sm[r][c], c counted from X0 - HX
    const float(*sm)[BW] = reinterpret_cast<const float(*)[BW]>(&sbox[0][CX]);

    if constexpr (CFG) {
        // score of every pixel of the tile and its 1-pixel ring; pixels within
        // 3 of the level edge (and outside the level) are never corners
        for (int i = t; i < (TH + 2) * (TW + 2); i += K1_THREADS) {
            const int sr = i / (TW + 2), sc = i - sr * (TW + 2);
            const int y = Y0 - 1 + sr, x = X0 - 1 + sc;
            uint32_t arc = 0u;
            float score = 0.0f;
            if (y >= 3 && y < h - 3 && x >= 3 && x < w - 3) score = cfg_corner(sm, sr - 1 + HY, sc - 1 + HX, &arc);
            s_score[sr][sc] = score;
            s_arc[sr][sc] = (uint8_t)arc;
        }
        __syncthreads();
    }

    const int tx = t % TW;
    const int x = X0 + tx;
    if (x >= w) return;
    // blur taps, x part (this thread's column is fixed)
    int ix0[3], ix1[3];
    float ax[3];
    {
        const float uvx = ((float)x + 0.5f) * tex_x;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float u = (uvx + off[k] * tex_x) * (float)w - 0.5f;
            const float fi = floorf(u);
            ax[k] = u - fi;
            int c0 = edge_index(fi, w) - (X0 - HX), c1 = edge_index(fi + 1.0f, w) - (X0 - HX);
            if (c0 < 0 || c1 >= SW) atomicOr(err, USLAM_ERR_SMEM_RANGE);
            ix0[k] = min(max(c0, 0), SW - 1);
            ix1[k] = min(max(c1, 0), SW - 1);
        }
    }
    // the column taps of an interior column sit at -2, -1 | d, d + 1 | 1, 2
    // around the pixel (d = dcx = -1 or 0): no edge clamp (warp-uniform flag)
    const int cc = tx + HX, dcx = ix0[1] - cc;
    const bool colfast = __all_sync(__activemask(), ix0[0] == cc - 2 && ix1[0] == cc - 1 && (dcx == -1 || dcx == 0) &&
                                                        ix1[1] == ix0[1] + 1 && ix0[2] == cc + 1 && ix1[2] == cc + 2);
    const uint32_t* mask = F.mask[l];
    uint8_t* const kpmap = F.kpmap[l];
    float* const blur = F.blur[l];
    const int kp_pitch = F.kp_pitch[l], bl_pitch = F.bl_pitch[l];
    // x weights of the taps as pairs: (a_i, a_i) and (1 - a_i, 1 - a_i) for
    // the pairs (i, j = 0 | 1), and (a_0, a_1), (1 - a_0, 1 - a_1) for the pair
    // (i = 0 | 1, j = 2); tap weights 0.3125, 0.375, 0.3125
    float2 pa[3], pna[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        pa[i] = make_float2(ax[i], ax[i]);
        pna[i] = make_float2(1.0f - ax[i], 1.0f - ax[i]);
    }
    const float2 pa01 = make_float2(ax[0], ax[1]);
    const float2 pna01 = make_float2(1.0f - ax[0], 1.0f - ax[1]);
    const float2 wt_same[3] = {make_float2(0.3125f, 0.3125f), make_float2(0.375f, 0.375f),
                               make_float2(0.3125f, 0.3125f)};
    const float2 wt01 = make_float2(0.3125f, 0.375f);
    for (int ty = t / TW; ty < TH; ty += K1_THREADS / TW) {
        const int y = Y0 + ty;
        if (y >= h) break;
        const int r = ty + HY, c = tx + HX;
        const size_t p = (size_t)y * (size_t)w + (size_t)x;

        uint32_t keep = 0;
        if constexpr (CFG) {
            // 3x3 NMS on the score; a tie goes to the first pixel in raster order
            const uint32_t A = s_arc[ty + 1][tx + 1];
            if (A) {
                const float Sc = s_score[ty + 1][tx + 1];
                bool ok = true;
#pragma unroll
                for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                    for (int dx = -1; dx <= 1; ++dx) {
                        if (dy == 0 && dx == 0) continue;
                        const float q = s_score[ty + 1 + dy][tx + 1 + dx];
                        const bool earlier = dy < 0 || (dy == 0 && dx < 0);
                        ok = ok && (earlier ? (Sc > q) : (Sc >= q));
                    }
                keep = ok ? A : 0u;
            }
        } else {
            // 2. FAST response + cull (resources/cull_corners.wgsl; see mask_bit)
            const uint32_t S = fast_response(sm, r, c);
            if (S > 0u && mask_bit(mask, (int)p)) {
                keep = S;
                if (y == 0) {
                    // row 0: first arg-max of the 1x3 region [9k, min(9k+3, w))
                    const int start = x - x % 9;
                    const int end = min(start + 3, w);
                    for (int q = start; q < end; ++q) {
                        if (q == x) continue;
                        const uint32_t Sq = fast_response(sm, r, c + (q - x));
                        if ((q < x && Sq >= S) || (q > x && Sq > S)) keep = 0;
                    }
                }
            }
        }
        kpmap[(size_t)y * kp_pitch + x] = (uint8_t)keep;

        // 3. blur cache: G(x, y) of generate_features.wgsl:149-172.  Tap (i, j)
        // is sv = (na nb) T00 + (a nb) T10 + (na b) T01 + (a b) T11 summed
        // left to right, then q = (sv wt_i) wt_j, and G = the q summed j-major,
        // i-minor from 0.  The products of two taps run as packed pairs
        // ((i, 0) with (i, 1), and (0, 2) with (1, 2)); every lane is the scalar
        // product, and the sums are scalar in the written order.
        // texel(i, j, e, f): T of tap (i, j), e = row 0 / 1, f = column 0 / 1.
        const auto blur_value = [&](auto texel) -> float {
            float q[3][3];
            {
                const float2 b01 = s_b01[ty], nb01 = s_nb01[ty];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const float2 t00 = make_float2(texel(i, 0, 0, 0), texel(i, 1, 0, 0));
                    const float2 t10 = make_float2(texel(i, 0, 0, 1), texel(i, 1, 0, 1));
                    const float2 t01 = make_float2(texel(i, 0, 1, 0), texel(i, 1, 1, 0));
                    const float2 t11 = make_float2(texel(i, 0, 1, 1), texel(i, 1, 1, 1));
                    const float2 sv = sum4(mul2_rn(mul2_rn(pna[i], nb01), t00), mul2_rn(mul2_rn(pa[i], nb01), t10),
                                           mul2_rn(mul2_rn(pna[i], b01), t01), mul2_rn(mul2_rn(pa[i], b01), t11));
                    const float2 qq = mul2_rn(mul2_rn(sv, wt_same[i]), wt01);
                    q[0][i] = qq.x;
                    q[1][i] = qq.y;
                }
            }
            {
                const float2 b22 = s_b22[ty], nb22 = s_nb22[ty];
                const float2 t00 = make_float2(texel(0, 2, 0, 0), texel(1, 2, 0, 0));
                const float2 t10 = make_float2(texel(0, 2, 0, 1), texel(1, 2, 0, 1));
                const float2 t01 = make_float2(texel(0, 2, 1, 0), texel(1, 2, 1, 0));
                const float2 t11 = make_float2(texel(0, 2, 1, 1), texel(1, 2, 1, 1));
                const float2 sv = sum4(mul2_rn(mul2_rn(pna01, nb22), t00), mul2_rn(mul2_rn(pa01, nb22), t10),
                                       mul2_rn(mul2_rn(pna01, b22), t01), mul2_rn(mul2_rn(pa01, b22), t11));
                const float2 qq = mul2_rn(mul2_rn(sv, wt01), wt_same[2]);
                q[2][0] = qq.x;
                q[2][1] = qq.y;
                const float a = ax[2], na = pna[2].x, b = b22.x, nb = nb22.x;
                float s2 = (na * nb) * texel(2, 2, 0, 0);
                s2 = s2 + (a * nb) * texel(2, 2, 0, 1);
                s2 = s2 + (na * b) * texel(2, 2, 1, 0);
                s2 = s2 + (a * b) * texel(2, 2, 1, 1);
                q[2][2] = (s2 * 0.3125f) * 0.3125f;
            }
            float sum = 0.0f;
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int i = 0; i < 3; ++i) sum = sum + q[j][i];
            return sum;
        };
        float sum;
        if (colfast && s_rowfast[ty]) {
            // interior: the taps sit at rows / columns -2, -1 | d, d + 1 | 1, 2
            // around the pixel (d = -1 or 0, per column dcx, per row dry), so
            // every load is one of four base pointers plus a constant
            const float* P = &sm[r][c];
            const int dry = s_by0[1][ty] - r;
            const float* Px = P + dcx;
            const float* Py = P + dry * BW;
            const float* Pxy = Py + dcx;
            sum = blur_value([&](int i, int j, int e, int f) -> float {
                const float* base = i == 1 ? (j == 1 ? Pxy : Px) : (j == 1 ? Py : P);
                const int ro = (j == 0 ? -2 : (j == 1 ? 0 : 1)) + e;
                const int co = (i == 0 ? -2 : (i == 1 ? 0 : 1)) + f;
                return base[ro * BW + co];
            });
        } else {
            const float* row0[3];
            const float* row1[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                row0[j] = sm[s_by0[j][ty]];
                row1[j] = sm[s_by1[j][ty]];
            }
            sum = blur_value([&](int i, int j, int e, int f) -> float {
                return (e ? row1[j] : row0[j])[f ? ix1[i] : ix0[i]];
            });
        }
        blur[(size_t)y * bl_pitch + x] = sum;
    }
}

// ------------------------------------------------------------ compact ----
constexpr int KC_THREADS = 1024;

__device__ __forceinline__ int nonzero_bytes(uint32_t v) {
    return __popc(__vcmpne4(v, 0u)) >> 3;
}

// Block-wide exclusive scan of one value per thread; returns the prefix and
// writes the block total to *total.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t wv = lane < nwarps ? s_warp[lane] : 0u;
        uint32_t wi = wv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nwarps) s_warp[lane] = wi - wv;
        if (lane == 31) s_warp[32] = wi;
    }
    __syncthreads();
    const uint32_t res = s_warp[warp] + incl - v;
    *total = s_warp[32];
    __syncthreads();
    return res;
}

__device__ __forceinline__ void write_header(uint32_t* feats, uint32_t pos, int x, int y, uint32_t s) {
    uint32_t* rec = feats + (size_t)pos * 12u;
    rec[0] = __float_as_uint((float)x);
    rec[1] = __float_as_uint((float)y);
    rec[2] = s;
}

// One lane's 32-pixel row segment of a 32x32 cell (bytes at x >= w zeroed).
__device__ __forceinline__ void load_cell_row(const uint8_t* kp, int kpitch, int w, int h, int x0, int y,
                                              uint32_t v[8]) {
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = 0u;
    if (y >= h) return;
    const uint8_t* row = kp + (size_t)y * kpitch + x0;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (x0 + 16 * j < w) {  // then x0 + 16 j + 16 <= kpitch (a multiple of 16)
            const uint4 q = *reinterpret_cast<const uint4*>(row + 16 * j);
            v[4 * j] = q.x;
            v[4 * j + 1] = q.y;
            v[4 * j + 2] = q.z;
            v[4 * j + 3] = q.w;
        }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int rem = w - (x0 + 4 * k);
        if (rem <= 0) v[k] = 0u;
        else if (rem < 4) v[k] &= (1u << (8 * rem)) - 1u;
    }
}

__device__ void xsort_level(const FrameDev& F, int l, uint32_t kept, uint32_t* s_hist, uint32_t* s_warp);

// One counting-sort pass over a level's kept features (dynamic shared memory
// s_hist of w + 1 counters): the indices of the features with pick(i) true,
// sorted by x, go to order_out; colstart_out (if given) receives the first
// slot of each column.  Returns the number of features picked.
// inv_out (if given) receives for every picked feature i its position plus
// inv_base, and with inv_miss set ~0 for the others.
template <typename Pick>
__device__ uint32_t xsort_pass(const uint32_t* feats, uint32_t kept, int w, Pick pick, uint32_t* order_out,
                               uint32_t* colstart_out, uint32_t* s_hist, uint32_t* s_warp, uint32_t* inv_out = nullptr,
                               uint32_t inv_base = 0u, bool inv_miss = false) {
    for (int i = threadIdx.x; i <= w; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kept; i += blockDim.x)
        if (pick(i)) atomicAdd(&s_hist[(int)__uint_as_float(feats[(size_t)i * 12u])], 1u);
    __syncthreads();
    const int per = (w + (int)blockDim.x) / (int)blockDim.x;  // bins per thread over w + 1 bins
    const int b0 = threadIdx.x * per;
    uint32_t local = 0;
    for (int k = 0; k < per; ++k) {
        const int b = b0 + k;
        if (b < w) local += s_hist[b];
    }
    uint32_t tot;
    uint32_t run = block_exclusive_scan(local, s_warp, &tot);
    for (int k = 0; k < per; ++k) {
        const int b = b0 + k;
        if (b <= w) {
            const uint32_t c = b < w ? s_hist[b] : 0u;
            if (colstart_out) colstart_out[b] = run;
            s_hist[b] = run;  // becomes the fill cursor
            run += c;
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kept; i += blockDim.x) {
        if (pick(i)) {
            const uint32_t pos = atomicAdd(&s_hist[(int)__uint_as_float(feats[(size_t)i * 12u])], 1u);
            order_out[pos] = i;
            if (inv_out) inv_out[i] = inv_base + pos;
        } else if (inv_out && inv_miss) {
            inv_out[i] = 0xffffffffu;
        }
    }
    __syncthreads();
    return tot;
}

// LOD-0 y of a feature (match_features_cpu.cpp:58-64: f32 scale iterated).
__device__ __forceinline__ float lod0_y(const uint32_t* feats, uint32_t i, float scale) {
    return (float)(uint32_t)__uint_as_float(feats[(size_t)i * 12u + 1u]) * scale;
}

// The matcher's index of one level.  The frame height is cut into
// USLAM_MATCH_BANDS bands (LOD-0 rows [b H0 / B, (b + 1) H0 / B)):
//  * candidate list b = the features whose LOD-0 y lies in band b widened by
//    0.1 H0 + 2 (the window half-height plus slack), sorted by x, with the
//    first slot of each column; every feature inside the window of a query
//    of band b is in list b;
//  * query order = the features grouped by the band of their own LOD-0 y,
//    sorted by x within a band, with the band offsets after the column tables.
__device__ void xsort_level(const FrameDev& F, int l, uint32_t kept, uint32_t* s_hist, uint32_t* s_warp) {
    constexpr int NB = USLAM_MATCH_BANDS;
    const int w = F.w[l];
    const uint32_t* feats = F.feats[l];
    float scale = 1.0f;
    for (int i = 0; i < l; ++i) scale = scale * 1.2f;
    const float H = (float)(uint32_t)F.H0;
    const float margin = 0.1f * H + 2.0f;
    const size_t cap = (size_t)(F.cap > 0 ? F.cap : 1);
    uint32_t* qband = F.colstart[l] + (size_t)NB * (size_t)(w + 1);
    uint32_t* inv = F.winv[l];  // the tensor-core matcher's positions (null without it)
    for (int b = 0; b < NB; ++b) {
        const float lo = (float)b * H / (float)NB - margin, hi = (float)(b + 1) * H / (float)NB + margin;
        xsort_pass(
            feats, kept, w,
            [&](uint32_t i) {
                const float y = lod0_y(feats, i, scale);
                return y >= lo && y <= hi;
            },
            F.xorder[l] + (size_t)b * cap, F.colstart[l] + (size_t)b * (size_t)(w + 1), s_hist, s_warp,
            inv ? inv + cap * (size_t)(1 + b) : nullptr, 0u, true);
    }
    uint32_t base = 0;
    for (int b = 0; b < NB; ++b) {
        const uint32_t n = xsort_pass(
            feats, kept, w, [&](uint32_t i) { return match_band(lod0_y(feats, i, scale), H) == b; },
            F.qorder[l] + base, nullptr, s_hist, s_warp, inv, base, false);
        if (threadIdx.x == 0) qband[b] = base;
        base += n;
    }
    if (threadIdx.x == 0) qband[NB] = base;
}

// Per (frame, level): the x counting sort after the banded compaction.
__global__ void __launch_bounds__(KC_THREADS)
k_xsort(const FrameDev* __restrict__ frames, const SegDev* __restrict__ segs) {
    extern __shared__ uint32_t s_hist[];  // [w + 1]
    __shared__ uint32_t s_warp[33];
    const SegDev sg = segs[blockIdx.x];
    const FrameDev& F = frames[sg.frame];
    xsort_level(F, sg.level, F.kept[sg.level], s_hist, s_warp);
}

// --------------------------------------------------- banded compaction ----
// Keypoint compaction, spread over one CTA per 32-row band of every level (a
// band is also one row of 32x32 cells):
//   k_band_count  per band: raw keypoints and keypoints kept by the cell caps
//   k_band_write  per band: prefix of the earlier bands' kept counts, then the
//                 ordered write of the band's headers below the level cap;
//                 band 0 also writes the level's raw / kept totals
//   k_xsort       per level: counting sort of the kept features by x
// The list order ((y, x), or cell order with per-cell caps) is the band
// order followed by the order inside each band; the level cap keeps the
// first `cap` of it (generate_features.wgsl:67-70 appends in a racy order,
// so this canonical order is the deterministic policy).
constexpr int KBAND_THREADS = 256;
constexpr int KBAND_WARPS = KBAND_THREADS / 32;

// This warp's share of a band and its counts.  Rows mode: 4 rows per warp.
// Cells mode: a contiguous run of the band's cells per warp.
__device__ __forceinline__ void band_warp_counts(const FrameDev& F, int l, int band, uint32_t* raw, uint32_t* kept) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int w = F.w[l], h = F.h[l], kpitch = F.kp_pitch[l];
    const uint8_t* kp = F.kpmap[l];
    uint32_t r = 0, k = 0;
    if (F.cell_cap <= 0) {
        const int y0 = band * 32 + warp * (32 / KBAND_WARPS);
        for (int y = y0; y < min(h, y0 + 32 / KBAND_WARPS); ++y) {
            const uint32_t* row = reinterpret_cast<const uint32_t*>(kp + (size_t)y * kpitch);
            for (int x4 = lane; x4 * 4 < w; x4 += 32) r += nonzero_bytes(row[x4]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        k = r;
    } else {
        const uint32_t ccap = (uint32_t)F.cell_cap;
        const int ncx = (w + 31) / 32, per = (ncx + KBAND_WARPS - 1) / KBAND_WARPS;
        for (int cx = warp * per; cx < min(ncx, (warp + 1) * per); ++cx) {
            uint32_t v[8];
            load_cell_row(kp, kpitch, w, h, cx * 32, band * 32 + lane, v);
            uint32_t n = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) n += (uint32_t)nonzero_bytes(v[q]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
            r += n;
            k += n < ccap ? n : ccap;
        }
    }
    *raw = r;
    *kept = k;
}

__global__ void __launch_bounds__(KBAND_THREADS)
k_band_count(const FrameDev* __restrict__ frames, const BandItem* __restrict__ items) {
    __shared__ uint32_t s_raw[KBAND_WARPS], s_kept[KBAND_WARPS];
    const BandItem it = items[blockIdx.x];
    const FrameDev& F = frames[it.frame];
    uint32_t r, k;
    band_warp_counts(F, it.level, it.band, &r, &k);
    if ((threadIdx.x & 31) == 0) {
        s_raw[threadIdx.x >> 5] = r;
        s_kept[threadIdx.x >> 5] = k;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t R = 0, K = 0;
        for (int q = 0; q < KBAND_WARPS; ++q) {
            R += s_raw[q];
            K += s_kept[q];
        }
        F.bands[it.level][2 * it.band] = R;
        F.bands[it.level][2 * it.band + 1] = K;
    }
}

__global__ void __launch_bounds__(KBAND_THREADS)
k_band_write(const FrameDev* __restrict__ frames, const BandItem* __restrict__ items) {
    __shared__ uint32_t s_red[2][KBAND_WARPS];
    __shared__ uint32_t s_wbase[KBAND_WARPS];
    const BandItem it = items[blockIdx.x];
    const FrameDev& F = frames[it.frame];
    const int l = it.level, band = it.band;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int w = F.w[l], h = F.h[l], kpitch = F.kp_pitch[l];
    const uint8_t* kp = F.kpmap[l];
    const int nb = (h + 31) / 32;
    const uint32_t* bc = F.bands[l];
    uint32_t cap = (uint32_t)F.cap;
    if (F.frame_cap > 0) {
        // per-frame cap: what the earlier levels left of it (their kept
        // counts follow from their band counts, every level's being complete)
        uint32_t left = (uint32_t)F.frame_cap;
        for (int q = 0; q < l && left > 0u; ++q) {
            const int nbq = (F.h[q] + 31) / 32;
            uint32_t kq = 0;
            for (int b2 = lane; b2 < nbq; b2 += 32) kq += F.bands[q][2 * b2 + 1];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) kq += __shfl_xor_sync(0xffffffffu, kq, o);
            kq = min(kq, (uint32_t)F.cap);
            left -= min(kq, left);
        }
        cap = min(cap, left);
    }
    // prefix of the earlier bands' kept counts (band 0: also the level totals)
    uint32_t pk = 0, tr = 0, tk = 0;
    for (int q = threadIdx.x; q < nb; q += KBAND_THREADS) {
        const uint32_t kq = bc[2 * q + 1];
        if (q < band) pk += kq;
        tr += bc[2 * q];
        tk += kq;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pk += __shfl_xor_sync(0xffffffffu, pk, o);
        tr += __shfl_xor_sync(0xffffffffu, tr, o);
        tk += __shfl_xor_sync(0xffffffffu, tk, o);
    }
    if (lane == 0) {
        s_red[0][warp] = pk;
        s_red[1][warp] = tr;
    }
    __shared__ uint32_t s_tk[KBAND_WARPS];
    if (lane == 0) s_tk[warp] = tk;
    uint32_t r, k;
    band_warp_counts(F, l, band, &r, &k);
    if (lane == 0) s_wbase[warp] = k;
    __syncthreads();
    uint32_t prefix = 0;
    for (int q = 0; q < KBAND_WARPS; ++q) prefix += s_red[0][q];
    if (band == 0 && threadIdx.x == 0) {
        uint32_t R = 0, K = 0;
        for (int q = 0; q < KBAND_WARPS; ++q) {
            R += s_red[1][q];
            K += s_tk[q];
        }
        F.raw[l] = R;
        F.kept[l] = K < cap ? K : cap;
    }
    uint32_t running = prefix;
    for (int q = 0; q < warp; ++q) running += s_wbase[q];
    if (prefix >= cap) return;
    uint32_t* feats = F.feats[l];
    if (F.cell_cap <= 0) {
        const int y0 = band * 32 + warp * (32 / KBAND_WARPS);
        for (int y = y0; y < min(h, y0 + 32 / KBAND_WARPS); ++y) {
            const uint32_t* row = reinterpret_cast<const uint32_t*>(kp + (size_t)y * kpitch);
            for (int base = 0; base < w; base += 128) {
                const int x4 = base / 4 + lane;
                const uint32_t v = (x4 * 4 < w) ? row[x4] : 0u;
                const uint32_t n = (uint32_t)nonzero_bytes(v);
                uint32_t incl = n;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                uint32_t pos = running + incl - n;
                for (int b = 0; b < 4; ++b) {
                    const uint32_t sv = (v >> (8 * b)) & 0xffu;
                    if (sv == 0u) continue;
                    if (pos < cap) write_header(feats, pos, x4 * 4 + b, y, sv);
                    ++pos;
                }
                running += __shfl_sync(0xffffffffu, incl, 31);
            }
        }
    } else {
        const uint32_t ccap = (uint32_t)F.cell_cap;
        const int ncx = (w + 31) / 32, per = (ncx + KBAND_WARPS - 1) / KBAND_WARPS;
        const int y = band * 32 + lane;
        for (int cx = warp * per; cx < min(ncx, (warp + 1) * per); ++cx) {
            uint32_t v[8];
            load_cell_row(kp, kpitch, w, h, cx * 32, y, v);
            uint32_t n = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) n += (uint32_t)nonzero_bytes(v[q]);
            uint32_t incl = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
            uint32_t rank = incl - n;
            for (int q = 0; q < 8 && rank < ccap; ++q) {
                if (v[q] == 0u) continue;
                for (int b = 0; b < 4; ++b) {
                    const uint32_t sv = (v[q] >> (8 * b)) & 0xffu;
                    if (sv == 0u) continue;
                    if (rank < ccap && running + rank < cap) write_header(feats, running + rank, cx * 32 + 4 * q + b, y, sv);
                    ++rank;
                }
            }
            running += tot < ccap ? tot : ccap;
        }
    }
}

// ------------------------------------------------------------- K2 ----
constexpr int KD_THREADS = 256;
constexpr int MAX_SEGS = 4096;

// Prefix over per-segment counts, shared by the persistent kernels.
template <typename CountFn>
__device__ uint32_t segment_prefix(int nseg, uint32_t* s_pref, uint32_t* s_warp, CountFn count) {
    const int per = (nseg + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    uint32_t local = 0;
    for (int k = 0; k < per; ++k)
        if (b0 + k < nseg) local += count(b0 + k);
    uint32_t tot;
    uint32_t run = block_exclusive_scan(local, s_warp, &tot);
    for (int k = 0; k < per; ++k) {
        if (b0 + k < nseg) {
            s_pref[b0 + k] = run;
            run += count(b0 + k);
        }
    }
    if (threadIdx.x == 0) s_pref[nseg] = tot;
    __syncthreads();
    return tot;
}

__device__ __forceinline__ int find_segment(const uint32_t* s_pref, int nseg, uint32_t g) {
    int lo = 0, hi = nseg - 1;  // largest s with s_pref[s] <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_pref[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}


// Blur-cache border of one level: columns [w, w + M) and the negative-x
// sentinel column for rows [0, h), then rows [h, h + M) and the negative-y
// sentinel row for all columns.  A sentinel stands for every negative
// coordinate: u32(negative) converts to the same f32 2^32 for all offsets a
// BRIEF test can reach, so G is identical for all of them.
// Work units of one level's border: runs of 32 rows of the right margin
// (columns w .. w + M) and runs of 32 columns of the bottom margin (rows
// h .. h + M, all columns including the corner and the sentinel column).
__device__ __forceinline__ uint32_t border_units(const FrameDev& F, int l) {
    return (uint32_t)((F.h[l] + 31) / 32 + (F.w[l] + F.margin + 1 + 31) / 32);
}

// The blur cache beyond the level edges: G(P) of generate_features.wgsl:149-172
// for every border cell, with the operation sequence of k_detect's blur
// (canonical bilinear taps read from the level in global memory, coordinates
// clamped to the edge) and the x part of the 9 taps computed once per lane (a
// lane keeps one column and walks the rows of its unit).  Cells of the sentinel row / column use the
// u32-wrapped coordinate 0xffffffff that every negative coordinate becomes.
__global__ void __launch_bounds__(256)
k_blur_border(const FrameDev* __restrict__ frames, const SegDev* __restrict__ segs, int nseg) {
    __shared__ uint32_t s_pref[MAX_SEGS + 1];
    __shared__ uint32_t s_warp[33];
    __shared__ float s_lut[256];
    s_lut[threadIdx.x] = (float)threadIdx.x / 255.0f;
    const uint32_t total = segment_prefix(nseg, s_pref, s_warp, [&](int sg) {
        return border_units(frames[segs[sg].frame], segs[sg].level);
    });
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int nw = gridDim.x * (blockDim.x >> 5);
    const float off[3] = {-1.2f, 0.0f, 1.2f};
    const float wt[3] = {0.3125f, 0.375f, 0.3125f};
    for (uint32_t g = gw; g < total; g += nw) {
        const int sidx = find_segment(s_pref, nseg, g);
        const int unit = (int)(g - s_pref[sidx]);
        const FrameDev& F = frames[segs[sidx].frame];
        const int l = segs[sidx].level;
        const int w = F.w[l], h = F.h[l], M = F.margin, bp = F.bl_pitch[l];
        const int nr = (h + 31) / 32;
        int ex, ey0, ey1;
        bool active;
        if (unit < nr) {
            ex = w + lane;
            active = lane <= M;
            ey0 = unit * 32;
            ey1 = min(h, ey0 + 32);
        } else {
            ex = (unit - nr) * 32 + lane;
            active = ex <= w + M;
            ey0 = h;
            ey1 = h + M + 1;
        }
        if (!active) continue;
        const uint8_t* img = F.img;
        const int pitch = F.img_pitch;
        const float* lvl = l > 0 ? F.lvl[l] : nullptr;
        const int lp = F.lvl_pitch[l];
        const float tex_x = 1.0f / (float)w;
        const float tex_y = 1.0f / (float)h;
        const uint32_t px = ex < w + M ? (uint32_t)ex : 0xffffffffu;
        const float uvx = ((float)px + 0.5f) * tex_x;
        float ax[3];
        int ix0[3], ix1[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float u = (uvx + off[i] * tex_x) * (float)w - 0.5f;
            const float fi = floorf(u);
            ax[i] = u - fi;
            ix0[i] = edge_index(fi, w);
            ix1[i] = edge_index(fi + 1.0f, w);
        }
        float* out = F.blur[l];
        for (int ey = ey0; ey < ey1; ++ey) {
            const uint32_t py = ey < h + M ? (uint32_t)ey : 0xffffffffu;
            const float uvy = ((float)py + 0.5f) * tex_y;
            float sum = 0.0f;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float v = (uvy + off[j] * tex_y) * (float)h - 0.5f;
                const float fj = floorf(v);
                const float b = v - fj;
                const int j0 = edge_index(fj, h), j1 = edge_index(fj + 1.0f, h);
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    float t00, t10, t01, t11;
                    if (lvl) {
                        t00 = __ldg(lvl + (size_t)j0 * lp + ix0[i]);
                        t10 = __ldg(lvl + (size_t)j0 * lp + ix1[i]);
                        t01 = __ldg(lvl + (size_t)j1 * lp + ix0[i]);
                        t11 = __ldg(lvl + (size_t)j1 * lp + ix1[i]);
                    } else {
                        t00 = s_lut[__ldg(img + (size_t)j0 * pitch + ix0[i])];
                        t10 = s_lut[__ldg(img + (size_t)j0 * pitch + ix1[i])];
                        t01 = s_lut[__ldg(img + (size_t)j1 * pitch + ix0[i])];
                        t11 = s_lut[__ldg(img + (size_t)j1 * pitch + ix1[i])];
                    }
                    const float a = ax[i];
                    const float na = 1.0f - a, nb = 1.0f - b;
                    float sv = (na * nb) * t00;
                    sv = sv + (a * nb) * t10;
                    sv = sv + (na * b) * t01;
                    sv = sv + (a * b) * t11;
                    sum = sum + (sv * wt[i]) * wt[j];
                }
            }
            out[(size_t)ey * bp + ex] = sum;
        }
    }
}

// FP8 E4M3 code of an integer 0..16 (all exact: 2^k (1 + m / 8) with
// k = floor(log2 v) <= 4 and m = (v - 2^k) 8 / 2^k an integer).
__device__ __forceinline__ uint32_t e4m3_small_int(int v) {
    if (v <= 0) return 0u;
    const int k = 31 - __clz(v);
    return (uint32_t)(((k + 7) << 3) | (((v - (1 << k)) << 3) >> k));
}

// FP8 operand row of a descriptor (bit k -> 0x50 = 8.0 or 0x00) at row R of
// a K-major no-swizzle operand array: lane j writes bits 8 j .. 8 j + 7 (K
// chunk j / 2, half j % 2); wj = the descriptor word holding them.
__device__ __forceinline__ void write_fp8_row(uint8_t* base, uint32_t R, uint32_t wj, int lane) {
    const uint32_t bits = (wj >> (8 * (lane & 3))) & 0xffu;
    uint32_t lo = 0u, hi = 0u;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        lo |= ((bits >> b) & 1u) * (0x50u << (8 * b));
        hi |= ((bits >> (b + 4)) & 1u) * (0x50u << (8 * b));
    }
    *reinterpret_cast<uint2*>(base + (size_t)(R >> 3) * 2048u + (lane >> 1) * 128u + (R & 7u) * 16u + (lane & 1) * 8u) =
        make_uint2(lo, hi);
}
// Extension row (32 E4M3 values) at row R, lanes 0-3: the popcount pc split
// into 16 integers <= 16, then 256, grp split into two integers <= 16, then 1.
__device__ __forceinline__ void write_ext_row(uint8_t* base, uint32_t R, uint32_t pc, int grp, int lane) {
    uint32_t ext[2] = {0u, 0u};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int e = 8 * lane + k;  // extension value index 0..31
        uint32_t code = 0u;
        if (e < 16) code = e4m3_small_int(min(16, max(0, (int)pc - 16 * e)));
        else if (e == 16) code = 0x78u;  // 256
        else if (e == 17) code = e4m3_small_int(min(grp, 16));
        else if (e == 18) code = e4m3_small_int(max(grp - 16, 0));
        else if (e == 19) code = 0x38u;  // 1
        ext[k >> 2] |= code << (8 * (k & 3));
    }
    *reinterpret_cast<uint2*>(base + (size_t)(R >> 3) * 256u + (lane >> 1) * 128u + (R & 7u) * 16u + (lane & 1) * 8u) =
        make_uint2(ext[0], ext[1]);
}
// Query-order position k of level l -> its operand row (each band's queries
// from a multiple of 128 rows).
__device__ __forceinline__ uint32_t win_query_row(const uint32_t* qband, int l, int wq_rows, uint32_t k) {
    uint32_t off = (uint32_t)l * (uint32_t)wq_rows, b = 0;
    while (b + 1 < (uint32_t)USLAM_MATCH_BANDS && k >= qband[b + 1]) {
        off += (qband[b + 1] - qband[b] + 127u) / 128u * 128u;
        ++b;
    }
    return off + (k - qband[b]);
}

// Finish one keypoint's record (the warp holds its 8 descriptor words, lane
// k the word k of every lane): orientation and descriptor into the record
// (generate_features.wgsl:170-172), plus the tensor-core operand rows (PACK,
// WIN) of the matchers that take them.
template <bool PACK, bool WIN>
__device__ __forceinline__ void emit_feature(const FrameDev& F, int l, uint32_t i, int w, int y, float theta,
                                             const uint32_t (&words)[8], int lane) {
    uint32_t* rec = F.feats[l] + (size_t)i * 12u;
    uint32_t out = __float_as_uint(theta);
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (lane == 4 + k) out = words[k];
    if (lane >= 3 && lane < 12) rec[lane] = out;
    if constexpr (WIN) {
        uint32_t wj = words[0];
        uint32_t pc = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if ((lane >> 2) == k) wj = words[k];
            pc += (uint32_t)__popc(words[k]);
        }
        const uint32_t* inv = F.winv[l];
        const size_t cap = (size_t)(F.cap > 0 ? F.cap : 1);
        const uint32_t* qband = F.colstart[l] + (size_t)USLAM_MATCH_BANDS * (size_t)(w + 1);
        write_fp8_row(F.wq8, win_query_row(qband, l, F.wq_rows, __ldg(inv + i)), wj, lane);
#pragma unroll
        for (int b = 0; b < USLAM_MATCH_BANDS; ++b) {
            const uint32_t pos = __ldg(inv + cap * (size_t)(1 + b) + i);
            if (pos == 0xffffffffu) continue;
            const uint32_t R = (uint32_t)(USLAM_MATCH_BANDS * l + b) * (uint32_t)F.wc_rows + pos;
            write_fp8_row(F.wc8, R, wj, lane);
            if (lane < 4) write_ext_row(F.wcext, R, pc, (int)(pos & 31u), lane);
            else if (lane == 4) F.wcy[R] = (uint16_t)y;
            else if (lane == 5) F.wcid[R] = USLAM_PACK(l, i);
        }
    }
    if constexpr (PACK) {
        // tensor-core operand rows of this feature (flat index f over
        // the levels): lane j writes the FP8 values of descriptor bits
        // 8j .. 8j + 7 (8.0 or 0; K chunk j / 2, half j % 2); lanes 0-3
        // write the 32-value extension row: the popcount split into 16
        // integers <= 16, then 256, the row's index within its 32-row
        // group split into two integers <= 16, then 1, then zeros
        uint32_t f = i;
        for (int q = 0; q < l; ++q) f += F.kept[q];
        uint32_t wj = words[0];
        uint32_t pc = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if ((lane >> 2) == k) wj = words[k];
            pc += (uint32_t)__popc(words[k]);
        }
        const uint32_t bits = (wj >> (8 * (lane & 3))) & 0xffu;
        uint32_t lo = 0u, hi = 0u;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            lo |= ((bits >> b) & 1u) * (0x50u << (8 * b));
            hi |= ((bits >> (b + 4)) & 1u) * (0x50u << (8 * b));
        }
        *reinterpret_cast<uint2*>(F.bf8 + (size_t)(f >> 3) * 2048u + (lane >> 1) * 128u + (f & 7u) * 16u +
                                  (lane & 1) * 8u) = make_uint2(lo, hi);
        if (lane < 4) {
            uint32_t ext[2] = {0u, 0u};
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int e = 8 * lane + k;  // extension value index 0..31
                const int grp = (int)(f & 31u);
                uint32_t code = 0u;
                if (e < 16) code = e4m3_small_int(min(16, max(0, (int)pc - 16 * e)));
                else if (e == 16) code = 0x78u;  // 256
                else if (e == 17) code = e4m3_small_int(min(grp, 16));
                else if (e == 18) code = e4m3_small_int(max(grp - 16, 0));
                else if (e == 19) code = 0x38u;  // 1
                ext[k >> 2] |= code << (8 * (k & 3));
            }
            *reinterpret_cast<uint2*>(F.bfext + (size_t)(f >> 3) * 256u + (lane >> 1) * 128u + (f & 7u) * 16u +
                                      (lane & 1) * 8u) = make_uint2(ext[0], ext[1]);
        }
        if (lane == 0) {
            F.bfpop[f] = pc;
            F.bfid[f] = USLAM_PACK(l, i);
        }
    }
}

// PACK: also write the brute-force tensor-core matcher's operand rows of
// every feature (FrameDev::bf8 / bfext / bfpop / bfid).  WIN: the windowed
// tensor-core matcher's rows: the feature's query row (wq8) and its row in
// every candidate list that holds it (wc8, wcext, wcy, wcid), at the
// positions k_xsort recorded (winv).
template <bool PACK, bool WIN>
__global__ void __launch_bounds__(KD_THREADS)
k_describe(const FrameDev* __restrict__ frames, const SegDev* __restrict__ segs, int nseg,
           const int32_t* __restrict__ pattern) {
    // the test pattern as f32 (each coordinate converted once per CTA, exactly)
    __shared__ float4 s_pat[256];
    __shared__ uint32_t s_pref[MAX_SEGS + 1];
    __shared__ uint32_t s_warp[33];
    __shared__ float s_lut[256];
    // the r = 3 disc in (dy outer, dx inner) order as compile-time constants, so
    // the unrolled moment sum multiplies by immediates (same f32 operations)
    constexpr int8_t kdx[29] = {0, -2, -1, 0, 1, 2, -2, -1, 0, 1, 2, -3, -2, -1, 0, 1, 2, 3, -2, -1, 0, 1, 2, -2, -1, 0, 1, 2, 0};
    constexpr int8_t kdy[29] = {-3, -2, -2, -2, -2, -2, -1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 3};
    for (int i = threadIdx.x; i < 256; i += KD_THREADS) {
        s_pat[i] = make_float4((float)pattern[4 * i], (float)pattern[4 * i + 1], (float)pattern[4 * i + 2],
                               (float)pattern[4 * i + 3]);
        s_lut[i] = (float)i / 255.0f;
    }
    const uint32_t total = segment_prefix(nseg, s_pref, s_warp, [&](int s) {
        return frames[segs[s].frame].kept[segs[s].level];
    });
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (KD_THREADS / 32) + (threadIdx.x >> 5);
    const int nw = gridDim.x * (KD_THREADS / 32);
    // A warp takes G consecutive keypoints: lane j < G first computes the
    // orientation of keypoint j, then the warp runs the 256 tests of each in
    // turn with its position and angle broadcast from that lane.  Warps take
    // every nw-th group; k = the groups per warp at 32 keypoints each, and G
    // (<= 32) the group size that spreads the keypoints evenly over k groups
    // per warp, so that no warp runs a group more than the others.
    const uint32_t per_round = 32u * (uint32_t)nw;
    const uint32_t kq = (total + per_round - 1u) / per_round;
    const uint32_t G = kq ? (total + kq * (uint32_t)nw - 1u) / (kq * (uint32_t)nw) : 1u;
    for (uint32_t g0 = (uint32_t)gw * G; g0 < total; g0 += (uint32_t)nw * G) {
        // orientation (generate_features.wgsl:80-99): intensity moments over
        // the r = 3 disc, summed in the reference's order, then atan2
        int my_seg = 0;
        uint32_t my_idx = 0;
        float my_theta = 0.0f, my_s = 0.0f, my_c = 0.0f;
        if ((uint32_t)lane < G && g0 + lane < total) {
            my_seg = find_segment(s_pref, nseg, g0 + lane);
            my_idx = g0 + lane - s_pref[my_seg];
            const FrameDev& F = frames[segs[my_seg].frame];
            const int l = segs[my_seg].level;
            const int w = F.w[l], h = F.h[l];
            const uint32_t* rec = F.feats[l] + (size_t)my_idx * 12u;
            const int x = (int)__uint_as_float(rec[0]);
            const int y = (int)__uint_as_float(rec[1]);
            const float* lvl = F.lvl[l];
            const int lp = F.lvl_pitch[l];
            float m10 = 0.0f, m01 = 0.0f;
#pragma unroll
            for (int k = 0; k < 29; ++k) {
                const int cx = tint_clamp(x + kdx[k], w);
                const int cy = tint_clamp(y + kdy[k], h);
                const float v = l == 0 ? s_lut[__ldg(F.img + (size_t)cy * F.img_pitch + cx)]
                                       : __ldg(lvl + (size_t)cy * (size_t)lp + cx);
                m10 = m10 + (float)kdx[k] * v;
                m01 = m01 + (float)kdy[k] * v;
            }
            my_theta = uslam_atan2f(m01, m10);
            uslam_sincosf(my_theta, &my_s, &my_c);
        }
        const int nk = (int)min(G, total - g0);
        for (int kp = 0; kp < nk; ++kp) {
            const int sidx = __shfl_sync(0xffffffffu, my_seg, kp);
            const uint32_t i = __shfl_sync(0xffffffffu, my_idx, kp);
            const float theta = __shfl_sync(0xffffffffu, my_theta, kp);
            const float s = __shfl_sync(0xffffffffu, my_s, kp);
            const float c = __shfl_sync(0xffffffffu, my_c, kp);
            const FrameDev& F = frames[segs[sidx].frame];
            const int l = segs[sidx].level;
            const int w = F.w[l], h = F.h[l];
            uint32_t* rec = F.feats[l] + (size_t)i * 12u;
            const int x = (int)__uint_as_float(rec[0]);
            const int y = (int)__uint_as_float(rec[1]);

            // 256 tests, lane j owns tests j, j + 32, ..., j + 224: 16 independent
            // gathers from the blur cache (negative coordinates -> sentinel).
            const float* blur = F.blur[l];
            const int bp = F.bl_pitch[l];
            const int sx = w + F.margin, sy = h + F.margin;
            float ga[8], gb[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float4 t = s_pat[lane + 32 * k];
                const float fax = t.x, fay = t.y, fbx = t.z, fby = t.w;
                int xa = x + (int)rintf(fax * c - fay * s);
                int ya = y + (int)rintf(fax * s + fay * c);
                int xb = x + (int)rintf(fbx * c - fby * s);
                int yb = y + (int)rintf(fbx * s + fby * c);
                xa = xa < 0 ? sx : xa;
                ya = ya < 0 ? sy : ya;
                xb = xb < 0 ? sx : xb;
                yb = yb < 0 ? sy : yb;
                ga[k] = __ldg(blur + (size_t)ya * bp + xa);
                gb[k] = __ldg(blur + (size_t)yb * bp + xb);
            }
            uint32_t words[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) words[k] = __ballot_sync(0xffffffffu, ga[k] > gb[k]);
            emit_feature<PACK, WIN>(F, l, i, w, y, theta, words, lane);
        }
    }
}

// --------------------------------------------- K2 over staged tiles ----
// The same orientation and descriptor as k_describe, with the blur-cache
// samples read from shared memory: one CTA per item = (frame, level, 32-row
// band, chunk of KDT_CW columns).  One 2D TMA load stages the box of the
// blur cache that every test of the item's keypoints can reach (rows
// y0 - R .. y0 + 31 + R, columns x0 - RX .. x0 + KDT_CW - 1 + RX, R = margin
// - 1 >= the largest rotated test offset, RX = R rounded up to 4 so the box
// starts on a 16-byte boundary); cells at negative coordinates get the
// sentinel values the gather path reads for them.  The item's keypoints are
// those of the band's list range (the band order of the compaction) with x
// in the chunk, taken in rounds of up to KDT_THREADS.
constexpr int KDT_THREADS = 256;
constexpr int KDT_WARPS = KDT_THREADS / 32;

template <bool PACK, bool WIN>
__global__ void __launch_bounds__(KDT_THREADS)
k_describe_tiled(const FrameDev* __restrict__ frames, const BandItem* __restrict__ items,
                 const int32_t* __restrict__ pattern, uint32_t* err) {
    extern __shared__ __align__(128) float s_box[];  // [BH][BW] blur-cache box
    __shared__ float4 s_pat[256];
    __shared__ float s_lut[256];
    __shared__ uint32_t s_list[KDT_THREADS];
    __shared__ uint32_t s_wcount[KDT_WARPS];
    __shared__ uint32_t s_pos[2];
    __shared__ __align__(8) uint64_t s_bar;
    constexpr int8_t kdx[29] = {0, -2, -1, 0, 1, 2, -2, -1, 0, 1, 2, -3, -2, -1, 0, 1, 2, 3, -2, -1, 0, 1, 2, -2, -1, 0, 1, 2, 0};
    constexpr int8_t kdy[29] = {-3, -2, -2, -2, -2, -2, -1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 3};
    const BandItem it = items[blockIdx.x];
    const FrameDev& F = frames[it.frame];
    const int l = it.level, band = it.band;
    const int w = F.w[l], h = F.h[l], M = F.margin;
    const int R = M - 1, RX = (R + 3) & ~3;
    const int BW = KDT_CW + 2 * RX, BH = 32 + 2 * R;
    const int x0 = (int)it.pad2 * KDT_CW, y0 = band * 32;
    const int xs = x0 - RX, ys = y0 - R;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // the band's range of the level's list: after the kept counts of the
    // earlier bands, clipped by the level's kept count (the cap); the box is
    // loaded only for a band that keeps keypoints
    if (warp == 0) {
        uint32_t pk = 0;
        for (int q = lane; q < band; q += 32) pk += F.bands[l][2 * q + 1];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) pk += __shfl_xor_sync(0xffffffffu, pk, o);
        if (lane == 0) {
            const uint32_t kept = F.kept[l];
            const uint32_t b0 = min(pk, kept), b1 = min(pk + F.bands[l][2 * band + 1], kept);
            s_pos[0] = b0;
            s_pos[1] = b1;
            if (b1 > b0) {
                const void* tmap = static_cast<const char*>(F.tmaps) +
                                   (size_t)(l * USLAM_TMAPS_PER_LEVEL + USLAM_NUM_TILE_SHAPES) * USLAM_TMAP_BYTES;
                mbar_init(&s_bar, 1u);
                mbar_expect_tx(&s_bar, (uint32_t)(BW * BH * 4));
                tma_load_2d(s_box, tmap, xs, ys, &s_bar);
            }
        }
    }
    __syncthreads();  // range, barrier initialised
    if (s_pos[1] <= s_pos[0]) return;  // no keypoint in the band: nothing loaded
    // while the box is in flight: the pattern, the selection and the
    // orientations of the first round (they read the level, not the box)
    for (int i = t; i < 256; i += KDT_THREADS) {
        s_pat[i] = make_float4((float)pattern[4 * i], (float)pattern[4 * i + 1], (float)pattern[4 * i + 2],
                               (float)pattern[4 * i + 3]);
        s_lut[i] = (float)i / 255.0f;
    }
    const uint32_t pos0 = s_pos[0], pos1 = s_pos[1];
    const uint32_t* feats = F.feats[l];
    bool box_ready = false;
    for (uint32_t base = pos0; base < pos1; base += KDT_THREADS) {
        // this pass's keypoints with x in the chunk, in list order
        const uint32_t i = base + (uint32_t)t;
        bool sel = false;
        if (i < pos1) {
            const int x = (int)__uint_as_float(__ldg(feats + (size_t)i * 12u));
            sel = x >= x0 && x < x0 + KDT_CW;
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, sel);
        if (lane == 0) s_wcount[warp] = (uint32_t)__popc(bal);
        __syncthreads();  // also the pattern and the lookup table of the first round
        uint32_t off = 0, nsel = 0;
        for (int q = 0; q < KDT_WARPS; ++q) {
            off += q < warp ? s_wcount[q] : 0u;
            nsel += s_wcount[q];
        }
        if (sel) s_list[off + (uint32_t)__popc(bal & ((1u << lane) - 1u))] = i;
        __syncthreads();
        // warp q takes G consecutive keypoints of the list (G <= 32); lane j
        // first computes the orientation of keypoint j
        const uint32_t G = (nsel + KDT_WARPS - 1) / KDT_WARPS;
        const uint32_t g0 = (uint32_t)warp * G;
        const int nk = (int)min(G, nsel > g0 ? nsel - g0 : 0u);
        float my_theta = 0.0f, my_s = 0.0f, my_c = 0.0f;
        if (lane < nk) {
            // orientation (generate_features.wgsl:80-99): intensity moments over
            // the r = 3 disc, summed in the reference's order, then atan2
            const uint32_t* rec = feats + (size_t)s_list[g0 + lane] * 12u;
            const int x = (int)__uint_as_float(rec[0]);
            const int y = (int)__uint_as_float(rec[1]);
            const float* lvl = F.lvl[l];
            const int lp = F.lvl_pitch[l];
            float m10 = 0.0f, m01 = 0.0f;
#pragma unroll
            for (int k = 0; k < 29; ++k) {
                const int cx = tint_clamp(x + kdx[k], w);
                const int cy = tint_clamp(y + kdy[k], h);
                const float v = l == 0 ? s_lut[__ldg(F.img + (size_t)cy * F.img_pitch + cx)]
                                       : __ldg(lvl + (size_t)cy * (size_t)lp + cx);
                m10 = m10 + (float)kdx[k] * v;
                m01 = m01 + (float)kdy[k] * v;
            }
            my_theta = uslam_atan2f(m01, m10);
            uslam_sincosf(my_theta, &my_s, &my_c);
        }
        if (!box_ready) {
            // the box has landed; cells at negative coordinates get the
            // sentinel column (x = w + M) / row (y = h + M) that every
            // negative coordinate reads
            const bool landed = mbar_wait(&s_bar, 0u, kTmaWaitLimit);
            if (__syncthreads_or(!landed)) {
                if (t == 0) atomicOr(err, USLAM_ERR_TMA_TIMEOUT);
                mbar_wait(&s_bar, 0u, kTmaWaitLimit);  // the copy in flight lands before the box is left
                return;
            }
            if (xs < 0 || ys < 0) {
                const float* blur = F.blur[l];
                const int bp = F.bl_pitch[l];
                const int nx = max(-xs, 0), ny = max(-ys, 0);
                const int n = ny * BW + (BH - ny) * nx;
                for (int k = t; k < n; k += KDT_THREADS) {
                    int r, c;
                    if (k < ny * BW) {
                        r = k / BW;
                        c = k - r * BW;
                    } else {
                        const int q = k - ny * BW;
                        r = ny + q / nx;
                        c = q - (q / nx) * nx;
                    }
                    const int gy = ys + r, gx = xs + c;
                    if (gy > h + M || gx > w + M) continue;  // past the cache: never read by a test
                    s_box[r * BW + c] = blur[(size_t)(gy < 0 ? h + M : gy) * bp + (gx < 0 ? w + M : gx)];
                }
                __syncthreads();
            }
            box_ready = true;
        }
        for (int kp = 0; kp < nk; ++kp) {
            const uint32_t i2 = s_list[g0 + kp];
            const float theta = __shfl_sync(0xffffffffu, my_theta, kp);
            const float sn = __shfl_sync(0xffffffffu, my_s, kp);
            const float cs = __shfl_sync(0xffffffffu, my_c, kp);
            const uint32_t* rec = feats + (size_t)i2 * 12u;
            const int x = (int)__uint_as_float(rec[0]);
            const int y = (int)__uint_as_float(rec[1]);
            // 256 tests, lane j owns tests j, j + 32, ..., j + 224: 16 reads of
            // the staged box at (y + dy - ys, x + dx - xs)
            const float* org = s_box + (y - ys) * BW + (x - xs);
            float ga[8], gb[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float4 tp = s_pat[lane + 32 * k];
                const int xa = (int)rintf(tp.x * cs - tp.y * sn);
                const int ya = (int)rintf(tp.x * sn + tp.y * cs);
                const int xb = (int)rintf(tp.z * cs - tp.w * sn);
                const int yb = (int)rintf(tp.z * sn + tp.w * cs);
                ga[k] = org[ya * BW + xa];
                gb[k] = org[yb * BW + xb];
            }
            uint32_t words[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) words[k] = __ballot_sync(0xffffffffu, ga[k] > gb[k]);
            emit_feature<PACK, WIN>(F, l, i2, w, y, theta, words, lane);
        }
        __syncthreads();  // s_list / s_wcount reused by the next pass
    }
    if (!box_ready) mbar_wait(&s_bar, 0u, kTmaWaitLimit);  // no keypoint in the chunk: the load lands first
}

// Dynamic shared memory of k_describe_tiled for a blur-cache margin M (0 if
// the box would exceed a TMA box's 256 cells per dimension).
size_t describe_tiled_smem(int margin) {
    const int R = margin - 1, RX = (R + 3) & ~3;
    const int BW = KDT_CW + 2 * RX, BH = 32 + 2 * R;
    if (R < 0 || BW > 256 || BH > 256) return 0;
    return (size_t)BW * (size_t)BH * 4u;
}

// ------------------------------------------------- Hamming distance ----
// popcount(a ^ b) over 256 bits with 4 POPC instead of 8: three carry-save
// adders fold x0..x6 into ones (o3) and twos (t1, t2, t3), a fourth folds
// the twos into twos (tw) and fours (f); x7 is added as ones.  Per bit
// position x0 + .. + x7 = o3 + x7 + 2 tw + 4 f, so the sum of the weighted
// popcounts is the exact distance (integer arithmetic, no rounding).
// POPC issues at a quarter of the ALU rate, so this trades 4 POPC for
// 8 LOP3.
__device__ __forceinline__ uint32_t hamming256(const uint4& a0, const uint4& a1, const uint4& b0, const uint4& b1) {
    const uint32_t x0 = a0.x ^ b0.x, x1 = a0.y ^ b0.y, x2 = a0.z ^ b0.z, x3 = a0.w ^ b0.w;
    const uint32_t x4 = a1.x ^ b1.x, x5 = a1.y ^ b1.y, x6 = a1.z ^ b1.z, x7 = a1.w ^ b1.w;
    const uint32_t o1 = x0 ^ x1 ^ x2, t1 = (x0 & x1) | (x2 & (x0 ^ x1));
    const uint32_t o2 = o1 ^ x3 ^ x4, t2 = (o1 & x3) | (x4 & (o1 ^ x3));
    const uint32_t o3 = o2 ^ x5 ^ x6, t3 = (o2 & x5) | (x6 & (o2 ^ x5));
    const uint32_t tw = t1 ^ t2 ^ t3, f = (t1 & t2) | (t3 & (t1 ^ t2));
    return (uint32_t)__popc(o3) + (uint32_t)__popc(x7) + 2u * (uint32_t)__popc(tw) + 4u * (uint32_t)__popc(f);
}

// ------------------------------------------------------------- K3 ----
constexpr int KM_THREADS = 256;
// k_match CTAs resident per SM: registers up to 85 a thread (no spills);
// measured faster than 4 CTAs at 64 registers (0.584 against 0.633 ms on
// the 64-frame step) and than 2 at 128.
constexpr int KM_CTAS_PER_SM = 3;

struct MatchSegDev {
    int pair;
    int dir;    // tensor-core form: 0 queries = curr (b), pool = prev (a); 1 the reverse.
                // k_match searches both directions from the prev queries and ignores it.
    int level;
};

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

// First xb in [0, w] with fl(fl(xb * s) + d) >= c (w if none): the first
// column of a list whose features have LOD-0 x = c inside their own window
// (the b -> a test of match_features_cpu.cpp:106-115 seen from a).
__device__ int first_col_reach(float c, float d, float s, int w) {
    int xb = (int)fminf(fmaxf(floorf((c - d) / s) - 1.0f, 0.0f), (float)w);
    while (xb > 0 && (float)(xb - 1) * s + d >= c) --xb;
    while (xb < w && !((float)xb * s + d >= c)) ++xb;
    return xb;
}

// Last xb in [-1, w - 1] with fl(fl(xb * s) - d) <= c (-1 if none).
__device__ int last_col_reach(float c, float d, float s, int w) {
    int xb = (int)fminf(fmaxf(floorf((c + d) / s) + 1.0f, -1.0f), (float)(w - 1));
    while (xb < w - 1 && (float)(xb + 1) * s - d <= c) ++xb;
    while (xb >= 0 && !((float)xb * s - d <= c)) --xb;
    return xb;
}

// Lane-wise minimum / maximum of two 16-bit keys per word.
__device__ __forceinline__ uint32_t min_u16x2(uint32_t a, uint32_t b) {
    uint32_t r;
    asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}
__device__ __forceinline__ uint32_t max_u16x2(uint32_t a, uint32_t b) {
    uint32_t r;
    asm("max.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}

// Bits [lo, hi) of a staged batch that starts at list position base.
__device__ __forceinline__ uint32_t range_bits(uint32_t lo, uint32_t hi, uint32_t base) {
    const int a = (int)(max(lo, base) - base);
    const int b = (int)(min(hi, base + 32u) > base ? min(hi, base + 32u) - base : 0u);
    const uint32_t lo_mask = a >= 32 ? 0u : (0xffffffffu << a);
    const uint32_t hi_mask = b >= 32 ? 0xffffffffu : ((1u << b) - 1u);
    return lo_mask & hi_mask;
}

// One warp's staging area: 32 candidates (LOD-0 y, packed (level, index),
// descriptor halves), the packed (level, index) of each lane's query, and the
// batch's column keys: col[t * 32 + lane] = distance << 5 | lane for a hit of
// slot t by lane, all ones otherwise.
struct CandBuf {
    float py[32];
    int32_t idx[32];
    uint4 d0[32], d1[32];
};
struct CandStage {
    CandBuf buf[2];
    uint32_t qid[32];
    uint16_t col[32 * 32];
};
constexpr int KM_MAX_SEGS = USLAM_MAX_MATCH_SEGS;

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Query groups of one (pair, level) segment: groups of 32 queries of the
// previous set, per band of its query order.
__device__ __forceinline__ uint32_t match_groups(const FrameDev* frames, const PairDev* pairs, const MatchSegDev& sg) {
    const FrameDev& Qf = frames[pairs[sg.pair].prev];
    const int ql = sg.level;
    const uint32_t* qb = Qf.colstart[ql] + (size_t)USLAM_MATCH_BANDS * (size_t)(Qf.w[ql] + 1);
    uint32_t n = 0;
    for (int b = 0; b < USLAM_MATCH_BANDS; ++b) n += (qb[b + 1] - qb[b] + 31u) / 32u;
    return n;
}

// Band of group grp of a segment (grp becomes the group within the band).
__device__ __forceinline__ int match_group_band(const uint32_t* qband, uint32_t* grp) {
    int band = 0;
    while (band + 1 < USLAM_MATCH_BANDS && *grp >= (qband[band + 1] - qband[band] + 31u) / 32u) {
        *grp -= (qband[band + 1] - qband[band] + 31u) / 32u;
        ++band;
    }
    return band;
}

// The claim order of k_match: query groups by estimated cost, costliest
// first, so that the launch does not end on a few long groups.  A group's
// cost follows the candidates it stages: the union of its x-windows in the
// band lists of its pool levels, bounded by its first and last query (the
// group is x-sorted).  KM_BUCKETS cost buckets of 64 candidates.  The claim
// block of a launch: [0] the claim counter, [1, 1 + KM_BUCKETS) the groups
// per bucket, then the buckets' write cursors, then the order; k_mutual
// zeroes the first KM_CLAIM_WORDS words after the launch.
constexpr int KM_BUCKETS = 64;
constexpr int KM_CLAIM_WORDS = 1 + 2 * KM_BUCKETS;

__device__ uint32_t match_group_cost(const FrameDev* frames, const PairDev* pairs, const MatchSegDev& sg,
                                     uint32_t grp) {
    const PairDev& P = pairs[sg.pair];
    const FrameDev& Q = frames[P.prev];
    const FrameDev& B = frames[P.curr];
    const int l = sg.level;
    const uint32_t* qband = Q.colstart[l] + (size_t)USLAM_MATCH_BANDS * (size_t)(Q.w[l] + 1);
    const int band = match_group_band(qband, &grp);
    const uint32_t k0 = qband[band] + grp * 32u, k1 = min(k0 + 31u, qband[band + 1] - 1u);
    const float ql = lod_scale(l);
    const float x0 = (float)(uint32_t)__uint_as_float(Q.feats[l][(size_t)__ldg(Q.qorder[l] + k0) * 12u]) * ql;
    const float x1 = (float)(uint32_t)__uint_as_float(Q.feats[l][(size_t)__ldg(Q.qorder[l] + k1) * 12u]) * ql;
    const float lo = x0 - P.max_dx, hi = x1 + P.max_dx;
    uint32_t n = 0;
    for (int k = 0; k < 3; ++k) {
        const int pl = k == 0 ? l : (k == 1 ? l - 1 : l + 1);
        if (pl < 0 || pl >= B.levels) continue;
        const float ps = lod_scale(pl);
        const int wpl = B.w[pl];
        const uint32_t* colstart = B.colstart[pl] + (size_t)band * (size_t)(wpl + 1);
        const int xlo = first_col_ge(lo, ps, wpl), xhi = last_col_le(hi, ps, wpl);
        if (xlo <= xhi) n += __ldg(colstart + xhi + 1) - __ldg(colstart + xlo);
    }
    return n;
}

// Pass 1: every group's cost bucket and the bucket sizes.
__global__ void __launch_bounds__(256)
k_match_rank(const FrameDev* __restrict__ frames, const PairDev* __restrict__ pairs,
             const MatchSegDev* __restrict__ segs, int nseg, uint32_t* claim, uint8_t* gbucket) {
    __shared__ uint32_t s_pref[KM_MAX_SEGS + 1];
    __shared__ uint32_t s_warp[33];
    const uint32_t total =
        segment_prefix(nseg, s_pref, s_warp, [&](int s) { return match_groups(frames, pairs, segs[s]); });
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int sidx = find_segment(s_pref, nseg, g);
        const uint32_t c = match_group_cost(frames, pairs, segs[sidx], g - s_pref[sidx]);
        const int b = KM_BUCKETS - 1 - (int)min(c >> 6, (uint32_t)(KM_BUCKETS - 1));
        gbucket[g] = (uint8_t)b;
        atomicAdd(claim + 1 + b, 1u);
    }
}

// Pass 2: the order, bucket by bucket (within a bucket in arrival order).
__global__ void __launch_bounds__(256) k_match_order(uint32_t* claim, const uint8_t* __restrict__ gbucket) {
    __shared__ uint32_t s_start[KM_BUCKETS + 1];
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int b = 0; b < KM_BUCKETS; ++b) {
            s_start[b] = run;
            run += claim[1 + b];
        }
        s_start[KM_BUCKETS] = run;
    }
    __syncthreads();
    const uint32_t total = s_start[KM_BUCKETS];
    uint32_t* cursor = claim + 1 + KM_BUCKETS;
    uint32_t* order = claim + KM_CLAIM_WORDS;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int b = gbucket[g];
        order[s_start[b] + atomicAdd(cursor + b, 1u)] = g;
    }
}

// The windowed mutual matcher (match_features_cpu.cpp:66-207), one Hamming
// distance per pair of features.  Both directions of FindMatches compare the
// same pairs: b in the window of a (a -> b, pool = the levels l - 1 .. l + 1
// of the current set) and a in the window of b (b -> a).  So the queries of a
// launch are the previous set's features alone, and every distance feeds
// both searches:
//  * a warp takes 32 queries a of one band that are consecutive in x (from
//    the query level's x order) and streams the union of their windows, level
//    by level of the pool, through shared memory, 32 candidates at a time
//    (asynchronous copies, one batch ahead);
//  * per lane two exact index ranges of the x-ordered list: [m0, m1), the b
//    inside a's window, and [n0, n1), the b whose window holds a (the same
//    features except where f32 rounding at the window's x edge differs);
//    the y test |ya - yb| <= 0.1 H0 is the same both ways;
//  * a lane keeps a's two smallest keys (distance << 5 | slot) in registers,
//    and writes the key distance << 5 | lane of each hit into the column of
//    its slot; after the batch lane t folds column t into b's two smallest
//    and merges them into b's accumulator in HBM (atomic minimum of
//    (distance, packed a), then of the second distance), where the batches
//    of every query group that meets b meet;
//  * a2b is written per query group; k_mutual reads b's accumulator.
// A tied best leaves the second distance equal to the best, which fails the
// ratio test, so no result depends on the order of the candidates or of the
// merges.  The pool rule (fewer than two candidates: no match) is applied to
// a here and to b in k_mutual.
__global__ void __launch_bounds__(KM_THREADS, KM_CTAS_PER_SM)
k_match(const FrameDev* __restrict__ frames, const PairDev* __restrict__ pairs,
        const MatchSegDev* __restrict__ segs, int nseg, uint32_t* claim_block) {
    __shared__ uint32_t s_pref[KM_MAX_SEGS + 1];
    __shared__ uint32_t s_warp[33];
    __shared__ __align__(16) CandStage s_stage[KM_THREADS / 32];
    // work units: groups of 32 queries of one band (band offsets follow the
    // query level's column tables)
    const uint32_t total =
        segment_prefix(nseg, s_pref, s_warp, [&](int s) { return match_groups(frames, pairs, segs[s]); });
    uint32_t* const next_group = claim_block;
    const uint32_t* const order = claim_block ? claim_block + KM_CLAIM_WORDS : nullptr;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int gw = blockIdx.x * (KM_THREADS / 32) + warp;
    const int nw = gridDim.x * (KM_THREADS / 32);
    CandStage& S = s_stage[warp];
    {
        // the column keys start empty; each column pass empties its column again
        uint4* c = reinterpret_cast<uint4*>(S.col);
        for (int k = lane; k < (int)(sizeof(S.col) / 16); k += 32) c[k] = make_uint4(~0u, ~0u, ~0u, ~0u);
        __syncwarp();
    }
    // Query groups cost very different amounts (the hits in their windows).
    // With a claim block (its counter zeroed before the launch, its order
    // written by k_match_rank / k_match_order) a warp claims the next group of
    // the order, costliest first, when it finishes one; without it warps take
    // every nw-th group.  Each group writes only its own queries' a2b entries and merges
    // into b's accumulators by atomic minima, so the order does not change
    // the result.
    auto claim = [&](uint32_t g) -> uint32_t {
        if (!next_group) return g + (uint32_t)nw;
        uint32_t n = 0;
        if (lane == 0) n = atomicAdd(next_group, 1u);
        return __shfl_sync(0xffffffffu, n, 0);
    };
    for (uint32_t c = next_group ? claim(0u) : (uint32_t)gw; c < total; c = claim(c)) {
        const uint32_t g = order ? __ldg(order + c) : c;
        const int sidx = find_segment(s_pref, nseg, g);
        uint32_t grp = g - s_pref[sidx];
        const MatchSegDev sg = segs[sidx];
        const PairDev& P = pairs[sg.pair];
        const FrameDev& Q = frames[P.prev];
        const FrameDev& B = frames[P.curr];
        const int l = sg.level;
        const uint32_t* qband = Q.colstart[l] + (size_t)USLAM_MATCH_BANDS * (size_t)(Q.w[l] + 1);
        const int band = match_group_band(qband, &grp);
        const uint32_t qk = qband[band] + grp * 32u + (uint32_t)lane;
        const bool valid = qk < qband[band + 1];
        const uint32_t qi = valid ? __ldg(Q.qorder[l] + qk) : 0u;
        const uint32_t* qrec = Q.feats[l] + (size_t)qi * 12u;
        const float ql = lod_scale(l);
        const float cx = (float)(uint32_t)__uint_as_float(qrec[0]) * ql;
        const float cy = (float)(uint32_t)__uint_as_float(qrec[1]) * ql;
        const uint4 qd0 = *reinterpret_cast<const uint4*>(qrec + 4);
        const uint4 qd1 = *reinterpret_cast<const uint4*>(qrec + 8);
        const float dx = P.max_dx, dy = P.max_dy;
        const float lo = cx - dx, hi = cx + dx;
        S.qid[lane] = (uint32_t)USLAM_PACK(l, qi);
        __syncwarp();

        // a's best / second-best as keys (distance << 5 | slot); a tie on the
        // best distance leaves second >> 5 == best >> 5, which fails the test
        uint32_t bestk = 0xffffffffu, secondk = 0xffffffffu;
        int32_t bidx = -1;
        const int L = B.levels;
        uint4* const bacc = P.bacc;
        const size_t capb = (size_t)(B.cap > 0 ? B.cap : 1);
        uint16_t* const colq = S.col + lane;  // this lane's key of slot t at colq[32 t]
        for (int k = 0; k < 3; ++k) {
            const int pl = k == 0 ? l : (k == 1 ? l - 1 : l + 1);
            if (pl < 0 || pl >= L) continue;
            const float ps = lod_scale(pl);
            const int wpl = B.w[pl];
            // the pool's candidate list of this band
            const uint32_t* colstart = B.colstart[pl] + (size_t)band * (size_t)(wpl + 1);
            uint32_t m0 = 0u, m1 = 0u, n0 = 0u, n1 = 0u;
            if (valid) {
                int xlo = first_col_ge(lo, ps, wpl), xhi = last_col_le(hi, ps, wpl);
                if (xlo <= xhi) {
                    m0 = __ldg(colstart + xlo);
                    m1 = __ldg(colstart + xhi + 1);
                }
                xlo = first_col_reach(cx, dx, ps, wpl);
                xhi = last_col_reach(cx, dx, ps, wpl);
                if (xlo <= xhi) {
                    n0 = __ldg(colstart + xlo);
                    n1 = __ldg(colstart + xhi + 1);
                }
            }
            // union over both ranges and the warp (lanes are x-sorted, so it is contiguous)
            uint32_t c0 = min(m0 < m1 ? m0 : 0xffffffffu, n0 < n1 ? n0 : 0xffffffffu);
            uint32_t c1 = max(m0 < m1 ? m1 : 0u, n0 < n1 ? n1 : 0u);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                c0 = min(c0, __shfl_xor_sync(0xffffffffu, c0, o));
                c1 = max(c1, __shfl_xor_sync(0xffffffffu, c1, o));
            }
            if (c0 >= c1) continue;
            const uint32_t* xorder = B.xorder[pl] + (size_t)band * (size_t)(B.cap > 0 ? B.cap : 1);
            const uint32_t* feats = B.feats[pl];
            // Candidates are staged by asynchronous copies one batch ahead,
            // into two buffers: batch i + 1's copies are issued before batch i
            // is used, and batch i + 2's list entry is loaded meanwhile.
            uint32_t jn = 0u;  // list entry of this lane's slot in the next batch
            {
                // prologue: batch 0 in flight, batch 1's list entry in hand
                const uint32_t k0 = c0 + (uint32_t)lane;
                if (k0 < c1) {
                    const uint32_t j = __ldg(xorder + k0);
                    const uint32_t* rec = feats + (size_t)j * 12u;
                    CandBuf& N = S.buf[0];
                    cp_async4(&N.py[lane], rec + 1);
                    cp_async16(&N.d0[lane], rec + 4);
                    cp_async16(&N.d1[lane], rec + 8);
                    N.idx[lane] = USLAM_PACK(pl, j);
                }
                cp_async_commit();
                if (k0 + 32u < c1) jn = __ldg(xorder + k0 + 32u);
            }
            int cur = 0;
            for (uint32_t base = c0; base < c1; base += 32u, cur ^= 1) {
                const uint32_t kk = base + (uint32_t)lane;
                CandBuf& SB = S.buf[cur];
                {
                    // the next batch's copies go out before this batch is used
                    const uint32_t kn = kk + 32u;
                    if (kn < c1) {
                        const uint32_t* rec = feats + (size_t)jn * 12u;
                        CandBuf& N = S.buf[cur ^ 1];
                        cp_async4(&N.py[lane], rec + 1);
                        cp_async16(&N.d0[lane], rec + 4);
                        cp_async16(&N.d1[lane], rec + 8);
                        N.idx[lane] = USLAM_PACK(pl, jn);
                    }
                    cp_async_commit();
                    if (kn + 32u < c1) jn = __ldg(xorder + kn + 32u);
                    cp_async_wait<1>();
                    // the staged word is the record's f32 y; the LOD-0 y as in
                    // match_features_cpu.cpp:58-64
                    if (kk < c1) SB.py[lane] = (float)(uint32_t)SB.py[lane] * ps;
                }
                __syncwarp();
                // y test of all 32 staged candidates (unrolled, float4 loads);
                // slots past the list's end lie outside both ranges
                uint32_t ymask = 0u;
                const float4* py4 = reinterpret_cast<const float4*>(SB.py);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 v = py4[q];
                    ymask |= (!(fabsf(cy - v.x) > dy) ? 1u : 0u) << (4 * q);
                    ymask |= (!(fabsf(cy - v.y) > dy) ? 1u : 0u) << (4 * q + 1);
                    ymask |= (!(fabsf(cy - v.z) > dy) ? 1u : 0u) << (4 * q + 2);
                    ymask |= (!(fabsf(cy - v.w) > dy) ? 1u : 0u) << (4 * q + 3);
                }
                const uint32_t h1 = ymask & range_bits(m0, m1, base);  // b in a's window
                const uint32_t h0 = ymask & range_bits(n0, n1, base);  // a in b's window
                const uint32_t prev = bestk;
                uint32_t hb = h1 & h0;
                if (hb) {
                    // the next hit's descriptor is read while this one's
                    // distance is computed
                    int t = 31 - __clz(hb);
                    hb ^= 1u << t;
                    uint4 c0d = SB.d0[t], c1d = SB.d1[t];
                    while (true) {
                        const int tn = hb ? 31 - __clz(hb) : t;
                        const uint4 n0d = SB.d0[tn], n1d = SB.d1[tn];
                        const uint32_t d = hamming256(c0d, c1d, qd0, qd1);
                        const uint32_t key = (d << 5) | (uint32_t)t;
                        secondk = min(secondk, max(bestk, key));
                        bestk = min(bestk, key);
                        colq[32 * t] = (uint16_t)((d << 5) | (uint32_t)lane);
                        if (!hb) break;
                        hb ^= 1u << tn;
                        t = tn;
                        c0d = n0d;
                        c1d = n1d;
                    }
                }
                // pairs inside one direction's window only (rare)
                uint32_t o1 = h1 & ~h0, o0 = h0 & ~h1;
                if (__any_sync(0xffffffffu, (o1 | o0) != 0u)) {
                    while (o1) {
                        const int t = 31 - __clz(o1);
                        o1 ^= 1u << t;
                        const uint32_t key = (hamming256(SB.d0[t], SB.d1[t], qd0, qd1) << 5) | (uint32_t)t;
                        secondk = min(secondk, max(bestk, key));
                        bestk = min(bestk, key);
                    }
                    while (o0) {
                        const int t = 31 - __clz(o0);
                        o0 ^= 1u << t;
                        colq[32 * t] = (uint16_t)((hamming256(SB.d0[t], SB.d1[t], qd0, qd1) << 5) | (uint32_t)lane);
                    }
                }
                if (bestk != prev) bidx = SB.idx[bestk & 31u];
                __syncwarp();
                // column pass: lane t folds the keys of slot t into the two
                // smallest (two 16-bit lanes at a time), empties the column
                // and merges the pair into b's accumulator
                if (kk < c1) {
                    uint4* colt = reinterpret_cast<uint4*>(S.col + 32 * lane);
                    uint32_t b2 = 0xffffffffu, s2 = 0xffffffffu;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint4 v = colt[q];
                        colt[q] = make_uint4(~0u, ~0u, ~0u, ~0u);
                        s2 = min_u16x2(s2, max_u16x2(b2, v.x));
                        b2 = min_u16x2(b2, v.x);
                        s2 = min_u16x2(s2, max_u16x2(b2, v.y));
                        b2 = min_u16x2(b2, v.y);
                        s2 = min_u16x2(s2, max_u16x2(b2, v.z));
                        b2 = min_u16x2(b2, v.z);
                        s2 = min_u16x2(s2, max_u16x2(b2, v.w));
                        b2 = min_u16x2(b2, v.w);
                    }
                    const uint32_t bl = b2 & 0xffffu, bh = b2 >> 16;
                    const uint32_t cb = min(bl, bh);
                    const uint32_t cs = min(max(bl, bh), min(s2 & 0xffffu, s2 >> 16));
                    if (cb != 0xffffu) {
                        const unsigned long long key =
                            ((unsigned long long)(cb >> 5) << 32) | (unsigned long long)S.qid[cb & 31u];
                        const int32_t id = SB.idx[lane];
                        uint4* acc = bacc + (size_t)USLAM_PACK_LEVEL(id) * capb + (size_t)USLAM_PACK_INDEX(id);
                        const unsigned long long old = atomicMin(reinterpret_cast<unsigned long long*>(acc), key);
                        // the larger of the old best and this best joins the
                        // second-best candidates
                        const uint32_t lose = (uint32_t)((old > key ? old : key) >> 32);
                        atomicMin(&acc->z, min(lose, cs == 0xffffu ? 0xffffffffu : cs >> 5));
                    }
                }
                __syncwarp();
            }
        }
        if (valid) {
            uint32_t pool = B.kept[l];
            if (l > 0) pool += B.kept[l - 1];
            if (l + 1 < L) pool += B.kept[l + 1];
            int32_t res = -1;
            if (pool >= 2u && bidx >= 0 && (float)(bestk >> 5) < 0.85f * (float)(secondk >> 5)) res = bidx;
            P.a2b[(size_t)l * Q.cap + qi] = res;
        }
    }
}

// b's accumulators start empty (all ones) before every k_match launch: one
// CTA per (pair, level of b).
__global__ void __launch_bounds__(256)
k_bacc_init(const FrameDev* __restrict__ frames, const PairDev* __restrict__ pairs, const SegDev* __restrict__ segs) {
    const int pi = segs[blockIdx.x].frame;  // pair index
    const int l = segs[blockIdx.x].level;
    const PairDev& P = pairs[pi];
    const FrameDev& B = frames[P.curr];
    const uint32_t n = B.kept[l];
    uint4* acc = P.bacc + (size_t)l * (size_t)(B.cap > 0 ? B.cap : 1);
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) acc[i] = make_uint4(~0u, ~0u, ~0u, ~0u);
}

// ----------------------------------------------------- brute force ----
constexpr int KB_THREADS = 128;  // two queries per thread: 256 queries per CTA
constexpr int KB_TILE = 256;     // train descriptors per shared-memory tile
static_assert(KB_TILE <= 256, "tile slots are packed into 8 bits of the top-2 keys");

// Level of flat index f given the per-level prefix pre[0..L] (pre[L] = total).
__device__ __forceinline__ int flat_level(const uint32_t* pre, int L, uint32_t f) {
    int l = 0;
    while (l + 1 < L && pre[l + 1] <= f) ++l;
    return l;
}

// Brute-force top-2 matching (the benchmark's `cfg` matcher): every feature
// of frame prev (all levels) against every feature of frame curr, Lowe test
// best < ratio * second in f32, no window and no cross-check.  One CTA holds
// 256 queries in registers and streams the train set through shared memory
// in tiles of 256 descriptors.  A tied best fails the ratio test, so the
// result does not depend on the scan order; a train set of fewer than two
// features gives no match (the pool rule of match_features_cpu.cpp:80-82).
// Result per query a in a2b: packed (level, index) of its match in curr, or -1.
__global__ void __launch_bounds__(KB_THREADS, 8)
k_bruteforce(const FrameDev* __restrict__ frames, const PairDev* __restrict__ pairs, const SegDev* __restrict__ psegs,
             int npairs, float ratio) {
    __shared__ uint32_t s_pref[MAX_SEGS + 1];
    __shared__ uint32_t s_warp[33];
    __shared__ uint4 s_d[2 * KB_TILE];
    __shared__ int32_t s_id[KB_TILE];
    __shared__ uint32_t s_qpre[USLAM_MAX_LEVELS + 1], s_tpre[USLAM_MAX_LEVELS + 1];
    const uint32_t total = segment_prefix(npairs, s_pref, s_warp, [&](int s) {
        const PairDev& P = pairs[psegs[s].frame];
        const FrameDev& A = frames[P.prev];
        uint32_t n = 0;
        for (int l = 0; l < A.levels; ++l) n += A.kept[l];
        return (n + 2u * KB_THREADS - 1u) / (2u * KB_THREADS) * (uint32_t)max(P.bf_splits, 1);
    });
    const int tid = threadIdx.x;
    for (uint32_t g = blockIdx.x; g < total; g += gridDim.x) {
        const int sidx = find_segment(s_pref, npairs, g);
        const PairDev& P = pairs[psegs[sidx].frame];
        const uint32_t nsplit = (uint32_t)max(P.bf_splits, 1);
        const uint32_t unit = g - s_pref[sidx];
        const uint32_t blk = unit / nsplit, split = unit - blk * nsplit;
        const FrameDev& A = frames[P.prev];
        const FrameDev& B = frames[P.curr];
        const int LA = A.levels, LB = B.levels;
        if (tid == 0) {
            uint32_t ra = 0, rb = 0;
            for (int l = 0; l <= USLAM_MAX_LEVELS; ++l) {
                s_qpre[l] = ra;
                s_tpre[l] = rb;
                if (l < LA) ra += A.kept[l];
                if (l < LB) rb += B.kept[l];
            }
        }
        __syncthreads();
        const uint32_t nq = s_qpre[LA], nt = s_tpre[LB];
        uint4 q0[2], q1[2];
        uint32_t best[2], second[2];
        int32_t bidx[2];
        int ql[2];
        uint32_t qi[2];
        bool qv[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t f = blk * 2u * KB_THREADS + 2u * tid + k;
            qv[k] = f < nq;
            ql[k] = qv[k] ? flat_level(s_qpre, LA, f) : 0;
            qi[k] = qv[k] ? f - s_qpre[ql[k]] : 0u;
            const uint32_t* rec = A.feats[ql[k]] + (size_t)qi[k] * 12u;
            q0[k] = qv[k] ? *reinterpret_cast<const uint4*>(rec + 4) : make_uint4(0, 0, 0, 0);
            q1[k] = qv[k] ? *reinterpret_cast<const uint4*>(rec + 8) : make_uint4(0, 0, 0, 0);
            best[k] = second[k] = 0xffffffffu;  // keys: distance << 8 | tile slot
            bidx[k] = -1;
        }
        // this unit's share of the train set: tiles [split T / S, (split + 1) T / S)
        const uint32_t ntiles = (nt + KB_TILE - 1) / KB_TILE;
        const uint32_t tb = split * ntiles / nsplit, te = (split + 1u) * ntiles / nsplit;
        const uint32_t t_end = min(nt, te * (uint32_t)KB_TILE);
        for (uint32_t t0 = tb * (uint32_t)KB_TILE; t0 < t_end; t0 += KB_TILE) {
            __syncthreads();
            for (int j = tid; j < KB_TILE; j += KB_THREADS) {
                const uint32_t f = t0 + (uint32_t)j;
                if (f < t_end) {
                    const int l = flat_level(s_tpre, LB, f);
                    const uint32_t i = f - s_tpre[l];
                    const uint32_t* rec = B.feats[l] + (size_t)i * 12u;
                    s_d[2 * j] = __ldg(reinterpret_cast<const uint4*>(rec + 4));
                    s_d[2 * j + 1] = __ldg(reinterpret_cast<const uint4*>(rec + 8));
                    s_id[j] = USLAM_PACK(l, i);
                }
            }
            __syncthreads();
            const int n = (int)min((uint32_t)KB_TILE, t_end - t0);
            const uint32_t prev0 = best[0], prev1 = best[1];
            for (int j = 0; j < n; ++j) {
                const uint4 d0 = s_d[2 * j], d1 = s_d[2 * j + 1];
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    // min/max on (distance << 8 | slot) keep the two smallest
                    // distances; a tie leaves second >> 8 == best >> 8
                    const uint32_t key = (hamming256(q0[k], q1[k], d0, d1) << 8) | (uint32_t)j;
                    second[k] = min(second[k], max(best[k], key));
                    best[k] = min(best[k], key);
                }
            }
            // resolve this tile's winners to packed ids before the tile is overwritten
            if (best[0] != prev0) bidx[0] = s_id[best[0] & 255u];
            if (best[1] != prev1) bidx[1] = s_id[best[1] & 255u];
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (!qv[k]) continue;
            const size_t q = (size_t)ql[k] * A.cap + qi[k];
            if (nsplit == 1u) {
                const int32_t res =
                    (nt >= 2u && bidx[k] >= 0 && (float)(best[k] >> 8) < ratio * (float)(second[k] >> 8)) ? bidx[k]
                                                                                                          : -1;
                P.a2b[q] = res;
            } else {
                // partial record of this split; the emit kernel merges the splits
                const size_t stride = (size_t)A.levels * A.cap;
                *reinterpret_cast<uint4*>(P.bf_part + (split * stride + q) * 4u) =
                    make_uint4(best[k], second[k], (uint32_t)bidx[k], 0u);
            }
        }
        __syncthreads();  // s_qpre / s_tpre are rewritten by the next work unit
    }
}

// ---------------------------------------------------------- mutual ----
constexpr int KU_THREADS = 256;

// One CTA per (pair, level of a): keep (a, b) iff b2a[b] == a, in a order
// (match_features_cpu.cpp:196-205).
// MUTUAL = false: every a with a2b[a] >= 0 is emitted (brute-force mode,
// which has no cross-check).
template <bool MUTUAL>
__global__ void __launch_bounds__(KU_THREADS)
k_mutual(const FrameDev* __restrict__ frames, const PairDev* __restrict__ pairs, const SegDev* __restrict__ segs,
         uint32_t* err, uint32_t* reset_word) {
    // k_match's claim counters for its next launch on this stream (k_mutual
    // always follows k_match, which has finished with them)
    if (reset_word && blockIdx.x == 0)
        for (int i = threadIdx.x; i < KM_CLAIM_WORDS; i += blockDim.x) reset_word[i] = 0u;
    __shared__ uint32_t s_warp[33];
    const int pi = segs[blockIdx.x].frame;  // pair index
    const int l = segs[blockIdx.x].level;
    const PairDev& P = pairs[pi];
    const FrameDev& A = frames[P.prev];
    const FrameDev& B = frames[P.curr];
    const uint32_t n = A.kept[l];
    uint32_t base = 0;
    for (uint32_t c0 = 0; c0 < n; c0 += KU_THREADS) {
        const uint32_t i = c0 + threadIdx.x;
        int32_t m = -1;
        bool ok = false;
        if (i < n) {
            if (!MUTUAL && P.bf_splits > 1) {
                // merge the brute-force splits: the two smallest distances of the
                // union of the splits' (best, second) pairs; a tie on the best
                // leaves second == best, which fails the ratio test
                uint32_t bd = 0xffffffffu, sd = 0xffffffffu;
                int32_t bi = -1;
                const size_t stride = (size_t)A.levels * A.cap;
                for (int sp = 0; sp < P.bf_splits; ++sp) {
                    const uint4 e = *reinterpret_cast<const uint4*>(P.bf_part +
                                                                    (sp * stride + (size_t)l * A.cap + i) * 4u);
                    const uint32_t b = e.x >> 8, c = e.y >> 8;
                    if (b < bd) {
                        sd = min(bd, c);
                        bd = b;
                        bi = (int32_t)e.z;
                    } else {
                        sd = min(sd, b);
                    }
                }
                uint32_t nt = 0;
                for (int q = 0; q < B.levels; ++q) nt += B.kept[q];
                m = (nt >= 2u && bi >= 0 && (float)bd < P.bf_ratio * (float)sd) ? bi : -1;
                P.a2b[(size_t)l * A.cap + i] = m;
            } else {
                m = P.a2b[(size_t)l * A.cap + i];
            }
            if (m >= 0) {
                const int bl = USLAM_PACK_LEVEL(m), bi = USLAM_PACK_INDEX(m);
                if (!MUTUAL) {
                    ok = true;
                } else if (P.bacc) {
                    // b's search from its accumulator (k_match): the pool rule
                    // over a's levels bl - 1 .. bl + 1, the ratio test, and
                    // its nearest a is this a
                    const uint4 e = P.bacc[(size_t)bl * B.cap + bi];
                    uint32_t pool = A.kept[bl];
                    if (bl > 0) pool += A.kept[bl - 1];
                    if (bl + 1 < A.levels) pool += A.kept[bl + 1];
                    ok = pool >= 2u && e.y != 0xffffffffu && (float)e.y < 0.85f * (float)e.z &&
                         e.x == (uint32_t)USLAM_PACK(l, i);
                } else {
                    ok = P.b2a[(size_t)bl * B.cap + bi] == USLAM_PACK(l, i);
                }
            }
        }
        uint32_t tot;
        const uint32_t pos = base + block_exclusive_scan(ok ? 1u : 0u, s_warp, &tot);
        if (ok) {
            if (pos < (uint32_t)P.max_matches_per_level) {
                int32_t* o = P.matches + ((size_t)l * P.max_matches_per_level + pos) * 4;
                o[0] = l;
                o[1] = (int32_t)i;
                o[2] = USLAM_PACK_LEVEL(m);
                o[3] = USLAM_PACK_INDEX(m);
            } else {
                atomicOr(err, USLAM_ERR_MATCH_OVERFLOW);
            }
        }
        base += tot;
    }
    if (threadIdx.x == 0) P.match_count[l] = base;
}

// ------------------------------------------------------- frame ingest ----
// The reference's f32 pixel rule (data/src/provider_base.cpp:121-124 stores
// u8 / 255): the byte back, exact for those values; others become p * 255
// clamped to [0, 255] (NaN to 0) and rounded half to even.  One thread per 4
// pixels of a row.
__global__ void __launch_bounds__(128) k_frame_from_f32(const float* __restrict__ src, int W, int H, uint8_t* __restrict__ dst, int dpitch) {
    const int x4 = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (4 * x4 >= W || y >= H) return;
    const float* row = src + (size_t)y * W;
    uint32_t packed = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = 4 * x4 + k;
        if (x >= W) break;
        float t = row[x] * 255.0f;
        t = t > 0.0f ? (t < 255.0f ? t : 255.0f) : 0.0f;
        packed |= (uint32_t)__float2int_rn(t) << (8 * k);
    }
    uint8_t* out = dst + (size_t)y * dpitch + 4 * x4;
    if (4 * x4 + 4 <= W) {
        *reinterpret_cast<uint32_t*>(out) = packed;  // dpitch and the row start are multiples of 16
    } else {
        for (int k = 0; 4 * x4 + k < W; ++k) out[k] = (uint8_t)(packed >> (8 * k));
    }
}

}  // namespace uslam

// ------------------------------------------------------------ launch ----
namespace uslam {

cudaError_t init_constants() { return cudaSuccess; }

template <bool CFG>
cudaError_t launch_detect_profile(const FrameDev* frames, const TileItem* tiles, int ntiles, int shape, uint32_t* err,
                                  cudaStream_t st) {
    switch (shape) {
        case 0: k_detect<64, 32, CFG><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles, shape, err); break;
        case 1: k_detect<128, 32, CFG><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles, shape, err); break;
        case 2: k_detect<64, 16, CFG><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles, shape, err); break;
        case 3: k_detect<32, 32, CFG><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles, shape, err); break;
        case 4: k_detect<128, 16, CFG><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles, shape, err); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
cudaError_t launch_pyramid(const FrameDev* frames, const TileItem* tiles, int ntiles, int shape, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    switch (shape) {
        case 0: k_pyramid<64, 32><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles); break;
        case 1: k_pyramid<128, 32><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles); break;
        case 2: k_pyramid<64, 16><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles); break;
        case 3: k_pyramid<32, 32><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles); break;
        case 4: k_pyramid<128, 16><<<ntiles, K1_THREADS, 0, st>>>(frames, tiles); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_detect(const FrameDev* frames, const TileItem* tiles, int ntiles, int shape, int detector,
                          uint32_t* err, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    return detector == 1 ? launch_detect_profile<true>(frames, tiles, ntiles, shape, err, st)
                         : launch_detect_profile<false>(frames, tiles, ntiles, shape, err, st);
}

cudaError_t launch_compact_banded(const FrameDev* frames, const BandItem* bands, int nbands, const SegDev* segs,
                                  int nseg, int max_w, cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    k_band_count<<<nbands, KBAND_THREADS, 0, st>>>(frames, bands);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_band_write<<<nbands, KBAND_THREADS, 0, st>>>(frames, bands);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_xsort<<<nseg, KC_THREADS, (size_t)(max_w + 1) * sizeof(uint32_t), st>>>(frames, segs);
    return cudaGetLastError();
}

cudaError_t launch_xsort(const FrameDev* frames, const SegDev* segs, int nseg, int max_w, cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    k_xsort<<<nseg, KC_THREADS, (size_t)(max_w + 1) * sizeof(uint32_t), st>>>(frames, segs);
    return cudaGetLastError();
}

cudaError_t launch_blur_border(const FrameDev* frames, const SegDev* segs, int nseg, int grid, cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    k_blur_border<<<grid, 256, 0, st>>>(frames, segs, nseg);
    return cudaGetLastError();
}

cudaError_t launch_describe(const FrameDev* frames, const SegDev* segs, int nseg, const int32_t* pattern,
                            int grid, bool pack, bool win, cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    if (pack) k_describe<true, false><<<grid, KD_THREADS, 0, st>>>(frames, segs, nseg, pattern);
    else if (win) k_describe<false, true><<<grid, KD_THREADS, 0, st>>>(frames, segs, nseg, pattern);
    else k_describe<false, false><<<grid, KD_THREADS, 0, st>>>(frames, segs, nseg, pattern);
    return cudaGetLastError();
}

cudaError_t launch_describe_tiled(const FrameDev* frames, const BandItem* items, int nitems, const int32_t* pattern,
                                  bool pack, bool win, int margin, uint32_t* err, cudaStream_t st) {
    if (nitems <= 0) return cudaSuccess;
    const size_t smem = describe_tiled_smem(margin);
    if (pack) k_describe_tiled<true, false><<<nitems, KDT_THREADS, smem, st>>>(frames, items, pattern, err);
    else if (win) k_describe_tiled<false, true><<<nitems, KDT_THREADS, smem, st>>>(frames, items, pattern, err);
    else k_describe_tiled<false, false><<<nitems, KDT_THREADS, smem, st>>>(frames, items, pattern, err);
    return cudaGetLastError();
}

cudaError_t set_describe_tiled_smem(int margin) {
    const int smem = (int)describe_tiled_smem(margin);
    cudaError_t e = cudaFuncSetAttribute(k_describe_tiled<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_describe_tiled<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_describe_tiled<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return e;
}

// k_match over all SMs (num_sms x its resident CTAs).
cudaError_t launch_match(const FrameDev* frames, const PairDev* pairs, const void* segs, int nseg, int num_sms,
                         cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    k_match<<<num_sms * KM_CTAS_PER_SM, KM_THREADS, 0, st>>>(frames, pairs, static_cast<const MatchSegDev*>(segs), nseg,
                                                              nullptr);
    return cudaGetLastError();
}
// The claim order (k_match_rank, k_match_order), then k_match claiming from
// it.  claim: a block of match_claim_words(max groups) words, its first
// KM_CLAIM_WORDS zero (k_mutual_reset zeroes them again after each launch);
// gbucket: max groups bytes.
size_t match_claim_words(size_t max_groups) { return KM_CLAIM_WORDS + max_groups; }
cudaError_t launch_match_dyn(const FrameDev* frames, const PairDev* pairs, const void* segs, int nseg, int num_sms,
                             uint32_t* claim, uint8_t* gbucket, cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    const MatchSegDev* ms = static_cast<const MatchSegDev*>(segs);
    k_match_rank<<<num_sms * 4, 256, 0, st>>>(frames, pairs, ms, nseg, claim, gbucket);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_match_order<<<num_sms, 256, 0, st>>>(claim, gbucket);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_match<<<num_sms * KM_CTAS_PER_SM, KM_THREADS, 0, st>>>(frames, pairs, ms, nseg, claim);
    return cudaGetLastError();
}

cudaError_t launch_bacc_init(const FrameDev* frames, const PairDev* pairs, const SegDev* segs, int nseg,
                             cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    k_bacc_init<<<nseg, 256, 0, st>>>(frames, pairs, segs);
    return cudaGetLastError();
}

cudaError_t launch_mutual(const FrameDev* frames, const PairDev* pairs, const SegDev* segs, int nseg,
                          uint32_t* err, cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    k_mutual<true><<<nseg, KU_THREADS, 0, st>>>(frames, pairs, segs, err, nullptr);
    return cudaGetLastError();
}
cudaError_t launch_mutual_reset(const FrameDev* frames, const PairDev* pairs, const SegDev* segs, int nseg,
                                uint32_t* err, uint32_t* next_group, cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    k_mutual<true><<<nseg, KU_THREADS, 0, st>>>(frames, pairs, segs, err, next_group);
    return cudaGetLastError();
}

cudaError_t launch_emit(const FrameDev* frames, const PairDev* pairs, const SegDev* segs, int nseg, uint32_t* err,
                        cudaStream_t st) {
    if (nseg <= 0) return cudaSuccess;
    k_mutual<false><<<nseg, KU_THREADS, 0, st>>>(frames, pairs, segs, err, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_bruteforce(const FrameDev* frames, const PairDev* pairs, const SegDev* psegs, int npairs,
                              float ratio, int grid, cudaStream_t st) {
    if (npairs <= 0) return cudaSuccess;
    k_bruteforce<<<grid, KB_THREADS, 0, st>>>(frames, pairs, psegs, npairs, ratio);
    return cudaGetLastError();
}

cudaError_t launch_frame_from_f32(const float* src, int W, int H, uint8_t* dst, int dpitch, cudaStream_t st) {
    if (W <= 0 || H <= 0) return cudaSuccess;
    const dim3 grid((W / 4 + 127) / 128 + 1, H);
    k_frame_from_f32<<<grid, 128, 0, st>>>(src, W, H, dst, dpitch);
    return cudaGetLastError();
}

cudaError_t set_compact_smem(int max_w) {
    const size_t smem = (size_t)(max_w + 1) * sizeof(uint32_t);
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(k_xsort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace uslam
