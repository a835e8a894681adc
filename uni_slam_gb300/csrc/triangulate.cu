// triangulate.cu — batched two-view triangulation: the pass after RANSAC.
//
// Restates TriangulateCPU::execute (wslam/src/pose_estimate_cpu/triangulate_cpu.cpp:342-513)
// for many frame pairs in one call.  The rows of a pair are its RANSAC
// inliers as LOD-0 pixels; a pair's rows are cut into chunks of TRI_ROWS, one
// CTA per chunk, and every phase ends in the pair's "last chunk": the CTA that
// takes the pair's final ticket (atomic after a fence) combines the chunk
// partials in chunk order, so results do not depend on scheduling and nothing
// waits on another CTA.
//
//   k_tri_rays        PixelToNormalised of both pixels (map_helpers_lods.hpp:41-76, 110-120):
//                     the reference's double operations in its order, so the rays equal its
//                     bits; last chunk: the centroids of NormalisingTransform (:48-75)
//   k_tri_spread      distances to the centroids; last chunk: the Hartley scales
//   k_tri_gram        the 9-vector of each row of the normalised 8-point system (:98-118)
//                     and A^T A; last chunk: its eigenvector of the smallest eigenvalue (the
//                     right singular vector JacobiSVD yields, up to sign), the equal-singular-
//                     value projection, de-normalisation (:126-141) and the four (R, t) of
//                     DecomposeEssential (:150-176)
//   k_tri_cheirality  rows x 4 candidates: the DLT point (TriangulatePoint, :184-209) as the
//                     right singular vector of its 4x4 system (one-sided Jacobi); points in
//                     front of both cameras; last chunk: the first candidate with the most
//                     (ScoreCandidate :257-278, execute :409-421)
//   k_tri_landmarks   depth range and mean reprojection error of the chosen pose (:446-486);
//                     last chunk: the stats (:488-494)
//
// Binary64 throughout, no contraction (--fmad=false).  The SVDs are computed by
// other algorithms than Eigen's, so the pose and points agree with the
// reference to rounding (the tests state the tolerance), not bit for bit; the
// undistorted rays are bit-exact.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "runtime_internal.h"

namespace {

constexpr int TRI_ROWS = 32;   // rows per chunk (one warp)
constexpr int TRI_PART = 48;   // doubles of partials per chunk (45 used by A^T A)

struct TriParams {
    double fu, fv, cu, cv, k1, k2, p1, p2;
    double max_reproj, min_depth, max_depth, tol;
    int iters;
    int total;  // rows of all pairs
};

struct TriChunk {
    int pair, begin, end, pad;
};

struct TriPairDev {
    int begin, n, nchunks, first_chunk;
    int failed;  // the result is final (fit failed or no candidate in front)
    int best;
    int in_front[4];
    double cen[4];    // centroid of prev (x, y) and curr (x, y) rays
    double scale[2];  // Hartley scale of prev, curr
    double cand[4][12];  // R row-major, t
};

// ---- small helpers ---------------------------------------------------------

// PixelToNormalised: (pixel - c) / f, then UndistortNormalised's fixed-point
// iteration with the reference's expression order.
__device__ __forceinline__ void pixel_to_normalised(double px, double py, const TriParams& P, double& ox,
                                                    double& oy) {
    const double dx0 = (px - P.cu) / P.fu;
    const double dy0 = (py - P.cv) / P.fv;
    double x = dx0, y = dy0;
    for (int i = 0; i < P.iters; ++i) {
        const double r2 = x * x + y * y;
        const double radial = 1.0 + P.k1 * r2 + P.k2 * r2 * r2;
        const double dxt = 2.0 * P.p1 * x * y + P.p2 * (r2 + 2.0 * x * x);
        const double dyt = P.p1 * (r2 + 2.0 * y * y) + 2.0 * P.p2 * x * y;
        const double nx = (dx0 - dxt) / radial;
        const double ny = (dy0 - dyt) / radial;
        const double ex = nx - x, ey = ny - y;
        const double step = sqrt(ex * ex + ey * ey);
        x = nx;
        y = ny;
        if (step < P.tol) break;
    }
    ox = x;
    oy = y;
}

// ProjectToPixel (triangulate_cpu.cpp:34-45) with DistortNormalised
// (map_helpers_lods.hpp:16-29); false where z <= 0 (the reference's NaN).
__device__ __forceinline__ bool project_to_pixel(double X, double Y, double Z, const TriParams& P, double& u,
                                                 double& v) {
    if (!(Z > 0.0)) return false;
    const double x = X / Z, y = Y / Z;
    const double r2 = x * x + y * y;
    const double radial = 1.0 + P.k1 * r2 + P.k2 * r2 * r2;
    const double dx = 2.0 * P.p1 * x * y + P.p2 * (r2 + 2.0 * x * x);
    const double dy = P.p1 * (r2 + 2.0 * y * y) + 2.0 * P.p2 * x * y;
    u = P.fu * (x * radial + dx) + P.cu;
    v = P.fv * (y * radial + dy) + P.cv;
    return isfinite(u) && isfinite(v);
}

// Rotation (c, s) that zeroes a_pq of a symmetric matrix: A' = J^T A J with
// J_pp = J_qq = c, J_pq = s, J_qp = -s.  Returns false where a_pq is
// negligible beside both diagonal entries (then a_pq is set to zero).
__device__ __forceinline__ bool jacobi_angle(double app, double aqq, double apq, double& c, double& s) {
    const double g = 100.0 * fabs(apq);
    if (apq == 0.0 || (fabs(app) + g == fabs(app) && fabs(aqq) + g == fabs(aqq))) return false;
    const double theta = (aqq - app) / (2.0 * apq);
    double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
    if (theta < 0.0) t = -t;
    c = 1.0 / sqrt(t * t + 1.0);
    s = t * c;
    return true;
}

template <int P, int Q>
__device__ __forceinline__ void sym3_rotate(double (&a)[3][3], double (&v)[3][3]) {
    double c, s;
    if (!jacobi_angle(a[P][P], a[Q][Q], a[P][Q], c, s)) {
        a[P][Q] = a[Q][P] = 0.0;
        return;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const double ap = a[P][j], aq = a[Q][j];
        a[P][j] = c * ap - s * aq;
        a[Q][j] = s * ap + c * aq;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double ap = a[i][P], aq = a[i][Q];
        a[i][P] = c * ap - s * aq;
        a[i][Q] = s * ap + c * aq;
    }
    a[P][Q] = a[Q][P] = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double vp = v[i][P], vq = v[i][Q];
        v[i][P] = c * vp - s * vq;
        v[i][Q] = s * vp + c * vq;
    }
}

// SVD of a 3x3 through the eigen-decomposition of E^T E (cyclic Jacobi):
// singular values descending, V's columns the eigenvectors, u_i = E v_i / |E v_i|
// for the two largest, u3 = u1 x u2 (so det U = +1).
__device__ void svd3(const double (&e)[3][3], double (&u)[3][3], double (&sv)[3], double (&v)[3][3]) {
    double a[3][3], w[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) a[i][j] = (e[0][i] * e[0][j] + e[1][i] * e[1][j]) + e[2][i] * e[2][j];
    for (int sweep = 0; sweep < 50; ++sweep) {
        if (a[0][1] == 0.0 && a[0][2] == 0.0 && a[1][2] == 0.0) break;
        sym3_rotate<0, 1>(a, w);
        sym3_rotate<0, 2>(a, w);
        sym3_rotate<1, 2>(a, w);
    }
    // order the eigenpairs by eigenvalue, descending
    int o[3] = {0, 1, 2};
    const double d[3] = {a[0][0], a[1][1], a[2][2]};
    if (d[o[1]] > d[o[0]]) { const int t = o[0]; o[0] = o[1]; o[1] = t; }
    if (d[o[2]] > d[o[1]]) { const int t = o[1]; o[1] = o[2]; o[2] = t; }
    if (d[o[1]] > d[o[0]]) { const int t = o[0]; o[0] = o[1]; o[1] = t; }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = 0; i < 3; ++i) v[i][k] = w[i][o[k]];
    double ev[3][3];  // E v_k
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = 0; i < 3; ++i) ev[i][k] = (e[i][0] * v[0][k] + e[i][1] * v[1][k]) + e[i][2] * v[2][k];
#pragma unroll
    for (int k = 0; k < 3; ++k) sv[k] = sqrt((ev[0][k] * ev[0][k] + ev[1][k] * ev[1][k]) + ev[2][k] * ev[2][k]);
    double u1[3], u2[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) u1[i] = sv[0] > 0.0 ? ev[i][0] / sv[0] : (i == 0 ? 1.0 : 0.0);
    // u2: E v2 made orthogonal to u1 (they are, up to rounding), normalised
    double d12 = (u1[0] * ev[0][1] + u1[1] * ev[1][1]) + u1[2] * ev[2][1];
#pragma unroll
    for (int i = 0; i < 3; ++i) u2[i] = ev[i][1] - d12 * u1[i];
    double n2 = sqrt((u2[0] * u2[0] + u2[1] * u2[1]) + u2[2] * u2[2]);
    if (!(n2 > 0.0)) {  // rank < 2: any unit vector orthogonal to u1
        const int m = fabs(u1[0]) < 0.9 ? 0 : 1;
        double ax[3] = {0, 0, 0};
        ax[m] = 1.0;
        d12 = u1[m];
#pragma unroll
        for (int i = 0; i < 3; ++i) u2[i] = ax[i] - d12 * u1[i];
        n2 = sqrt((u2[0] * u2[0] + u2[1] * u2[1]) + u2[2] * u2[2]);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) u2[i] /= n2;
    const double u3[3] = {u1[1] * u2[2] - u1[2] * u2[1], u1[2] * u2[0] - u1[0] * u2[2],
                          u1[0] * u2[1] - u1[1] * u2[0]};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        u[i][0] = u1[i];
        u[i][1] = u2[i];
        u[i][2] = u3[i];
    }
}

// Eigenvector of the smallest eigenvalue of the symmetric 9x9 in sA (padded
// to 10x10 with a decoupled index 9), by cyclic Jacobi over one warp: each
// round applies 5 disjoint rotations (round-robin pairing with index 9 held
// fixed), rows then columns, V accumulating.
__device__ void sym9_min_eigvec(double (*sA)[10], double (*sV)[10], double* out) {
    const int lane = threadIdx.x & 31;
    __shared__ double s_c[5], s_s[5];
    __shared__ int s_p[5], s_q[5], s_rot[5];
    __shared__ int s_done;
    for (int sweep = 0; sweep < 40; ++sweep) {
        if (lane == 0) {
            double off = 0.0, dia = 0.0;
            for (int i = 0; i < 9; ++i) {
                dia += sA[i][i] * sA[i][i];
                for (int j = i + 1; j < 9; ++j) off += sA[i][j] * sA[i][j];
            }
            s_done = off <= 1e-34 * dia;
        }
        __syncwarp();
        if (s_done) break;
        for (int round = 0; round < 9; ++round) {
            if (lane < 5) {
                int p = lane == 0 ? round : (round + lane) % 9;
                int q = lane == 0 ? 9 : (round + 9 - lane) % 9;
                if (p > q) { const int t = p; p = q; q = t; }
                double c = 1.0, s = 0.0;
                int rot = 0;
                if (q < 9) {
                    rot = jacobi_angle(sA[p][p], sA[q][q], sA[p][q], c, s) ? 1 : 0;
                    if (!rot) sA[p][q] = sA[q][p] = 0.0;
                }
                s_c[lane] = c;
                s_s[lane] = s;
                s_p[lane] = p;
                s_q[lane] = q;
                s_rot[lane] = rot;
            }
            __syncwarp();
            for (int t = lane; t < 50; t += 32) {  // rows of A: J^T A
                const int k = t / 10, j = t % 10;
                if (!s_rot[k]) continue;
                const int p = s_p[k], q = s_q[k];
                const double c = s_c[k], s = s_s[k];
                const double ap = sA[p][j], aq = sA[q][j];
                sA[p][j] = c * ap - s * aq;
                sA[q][j] = s * ap + c * aq;
            }
            __syncwarp();
            for (int t = lane; t < 100; t += 32) {  // columns of A and V: (.) J
                const int k = (t % 50) / 10, i = t % 10;
                if (!s_rot[k]) continue;
                double(*M)[10] = t < 50 ? sA : sV;
                const int p = s_p[k], q = s_q[k];
                const double c = s_c[k], s = s_s[k];
                const double ap = M[i][p], aq = M[i][q];
                M[i][p] = c * ap - s * aq;
                M[i][q] = s * ap + c * aq;
            }
            __syncwarp();
            if (lane < 5 && s_rot[lane]) sA[s_p[lane]][s_q[lane]] = sA[s_q[lane]][s_p[lane]] = 0.0;
            __syncwarp();
        }
    }
    int m = 0;
    for (int i = 1; i < 9; ++i)
        if (sA[i][i] < sA[m][m]) m = i;
    if (lane < 9) out[lane] = sV[lane][m];
    __syncwarp();
}

// Right singular vector of the smallest singular value of the 4x4 a
// (columns a[.][j]) by one-sided Jacobi (Hestenes): rotate column pairs until
// all are orthogonal; V accumulates; the answer is V's column of least norm.
__device__ __forceinline__ void null4(double (&a)[4][4], double (&x)[4]) {
    double v[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    for (int sweep = 0; sweep < 30; ++sweep) {
        bool rotated = false;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i + 1; j < 4; ++j) {
                double al = 0.0, be = 0.0, ga = 0.0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    al += a[k][i] * a[k][i];
                    be += a[k][j] * a[k][j];
                    ga += a[k][i] * a[k][j];
                }
                if (!(fabs(ga) > 1e-15 * sqrt(al * be))) continue;
                rotated = true;
                const double zeta = (be - al) / (2.0 * ga);
                double t = 1.0 / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                if (zeta < 0.0) t = -t;
                const double c = 1.0 / sqrt(1.0 + t * t);
                const double s = c * t;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const double ai = a[k][i], aj = a[k][j];
                    a[k][i] = c * ai - s * aj;
                    a[k][j] = s * ai + c * aj;
                    const double vi = v[k][i], vj = v[k][j];
                    v[k][i] = c * vi - s * vj;
                    v[k][j] = s * vi + c * vj;
                }
            }
        if (!rotated) break;
    }
    double best = 0.0;
    int m = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const double nj = ((a[0][j] * a[0][j] + a[1][j] * a[1][j]) + a[2][j] * a[2][j]) + a[3][j] * a[3][j];
        if (j == 0 || nj < best) {
            best = nj;
            m = j;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double xv = v[k][0];
#pragma unroll
        for (int j = 1; j < 4; ++j)
            if (j == m) xv = v[k][j];
        x[k] = xv;
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Ticket of the pair: true in the CTA that finishes the pair's phase last.
// Every thread that wrote partials has fenced before the block barrier.
__device__ __forceinline__ bool last_chunk(unsigned* ticket, int nchunks) {
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(ticket, 1u);
        s_last = t == static_cast<unsigned>(nchunks) - 1u;
        if (s_last) *ticket = 0u;  // ready for the next phase
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}

__device__ void write_empty_result(uslam_tri_result* r, int n, int cheirality) {
    for (int i = 0; i < 9; ++i) r->rotation[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int i = 0; i < 3; ++i) r->translation[i] = 0.0;
    r->mean_reprojection_error_px = 0.0;
    r->rotation_angle_rad = 0.0;
    r->input_matches = n;
    r->landmark_count = 0;
    r->cheirality_passes = cheirality;
    r->pose_recovered = 0;
}

// ---- phases -----------------------------------------------------------------

__global__ void __launch_bounds__(TRI_ROWS)
k_tri_rays(TriParams P, const TriChunk* __restrict__ chunks, TriPairDev* pairs, const double4_32a* __restrict__ px,
           double4_32a* __restrict__ rays, double* part, unsigned* tickets) {
    const TriChunk ch = chunks[blockIdx.x];
    const int r = ch.begin + static_cast<int>(threadIdx.x);
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    if (r < ch.end) {
        const double4_32a q = px[r];
        pixel_to_normalised(q.x, q.y, P, s0, s1);
        pixel_to_normalised(q.z, q.w, P, s2, s3);
        rays[r] = make_double4_32a(s0, s1, s2, s3);
    }
    s0 = warp_sum(s0);
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    s3 = warp_sum(s3);
    if (threadIdx.x == 0) {
        double* o = part + static_cast<size_t>(blockIdx.x) * TRI_PART;
        o[0] = s0;
        o[1] = s1;
        o[2] = s2;
        o[3] = s3;
    }
    TriPairDev* pd = pairs + ch.pair;
    if (!last_chunk(tickets + ch.pair, pd->nchunks)) return;
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int c = 0; c < pd->nchunks; ++c) s += __ldcg(part + static_cast<size_t>(pd->first_chunk + c) * TRI_PART + threadIdx.x);
        pd->cen[threadIdx.x] = s / static_cast<double>(pd->n);
    }
}

__global__ void __launch_bounds__(TRI_ROWS)
k_tri_spread(const TriChunk* __restrict__ chunks, TriPairDev* pairs, const double4_32a* __restrict__ rays, double* part,
             unsigned* tickets) {
    const TriChunk ch = chunks[blockIdx.x];
    TriPairDev* pd = pairs + ch.pair;
    const int r = ch.begin + static_cast<int>(threadIdx.x);
    double dp = 0.0, dc = 0.0;
    if (r < ch.end) {
        const double4_32a q = rays[r];
        const double ax = q.x - pd->cen[0], ay = q.y - pd->cen[1];
        const double bx = q.z - pd->cen[2], by = q.w - pd->cen[3];
        dp = sqrt(ax * ax + ay * ay);
        dc = sqrt(bx * bx + by * by);
    }
    dp = warp_sum(dp);
    dc = warp_sum(dc);
    if (threadIdx.x == 0) {
        double* o = part + static_cast<size_t>(blockIdx.x) * TRI_PART;
        o[0] = dp;
        o[1] = dc;
    }
    if (!last_chunk(tickets + ch.pair, pd->nchunks)) return;
    if (threadIdx.x < 2) {
        double s = 0.0;
        for (int c = 0; c < pd->nchunks; ++c) s += __ldcg(part + static_cast<size_t>(pd->first_chunk + c) * TRI_PART + threadIdx.x);
        const double mean = s / static_cast<double>(pd->n);
        pd->scale[threadIdx.x] = mean > 1e-12 ? 1.4142135623730951 / mean : 1.0;
    }
}

__global__ void __launch_bounds__(TRI_ROWS)
k_tri_gram(const TriChunk* __restrict__ chunks, TriPairDev* pairs, const double4_32a* __restrict__ rays, double* part,
           unsigned* tickets, uslam_tri_result* results) {
    __shared__ double s_row[TRI_ROWS][9];
    __shared__ double sA[10][10], sV[10][10];
    __shared__ double s_v[9];
    const TriChunk ch = chunks[blockIdx.x];
    TriPairDev* pd = pairs + ch.pair;
    const int lane = threadIdx.x;
    const int r = ch.begin + lane;
    {
        double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (r < ch.end) {
            const double4_32a q = rays[r];
            const double sp = pd->scale[0], sc = pd->scale[1];
            // normalise: T (x, y, 1) with T = [[s, 0, -s cx], [0, s, -s cy], [0, 0, 1]]
            const double xp = sp * q.x + -sp * pd->cen[0];
            const double yp = sp * q.y + -sp * pd->cen[1];
            const double xc = sc * q.z + -sc * pd->cen[2];
            const double yc = sc * q.w + -sc * pd->cen[3];
            a[0] = xc * xp;
            a[1] = xc * yp;
            a[2] = xc;
            a[3] = yc * xp;
            a[4] = yc * yp;
            a[5] = yc;
            a[6] = xp;
            a[7] = yp;
            a[8] = 1.0;
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) s_row[lane][k] = a[k];
    }
    __syncwarp();
    double* o = part + static_cast<size_t>(blockIdx.x) * TRI_PART;
    for (int e = lane; e < 45; e += 32) {  // upper triangle (i <= j), row-major
        int i = 0, rem = e;
        while (rem >= 9 - i) {
            rem -= 9 - i;
            ++i;
        }
        const int j = i + rem;
        double s = 0.0;
        for (int k = 0; k < TRI_ROWS; ++k) s += s_row[k][i] * s_row[k][j];
        o[e] = s;
    }
    if (!last_chunk(tickets + ch.pair, pd->nchunks)) return;
    for (int e = lane; e < 100; e += 32) {
        (&sA[0][0])[e] = 0.0;
        (&sV[0][0])[e] = (e / 10 == e % 10) ? 1.0 : 0.0;
    }
    __syncwarp();
    for (int e = lane; e < 45; e += 32) {
        int i = 0, rem = e;
        while (rem >= 9 - i) {
            rem -= 9 - i;
            ++i;
        }
        const int j = i + rem;
        double s = 0.0;
        for (int c = 0; c < pd->nchunks; ++c) s += __ldcg(part + static_cast<size_t>(pd->first_chunk + c) * TRI_PART + e);
        sA[i][j] = s;
        sA[j][i] = s;
    }
    __syncwarp();
    sym9_min_eigvec(sA, sV, s_v);
    if (lane != 0) return;

    // e_norm (row-major fill of v), projected to two equal singular values
    double en[3][3], u[3][3], sv[3], v[3][3];
    for (int i = 0; i < 9; ++i) en[i / 3][i % 3] = s_v[i];
    svd3(en, u, sv, v);
    const double avg = 0.5 * (sv[0] + sv[1]);
    double ec[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) ec[i][j] = avg * (u[i][0] * v[j][0]) + avg * (u[i][1] * v[j][1]);
    // e_final = T_curr^T e_clean T_prev
    const double sp = pd->scale[0], sc = pd->scale[1];
    const double tp[3][3] = {{sp, 0.0, -sp * pd->cen[0]}, {0.0, sp, -sp * pd->cen[1]}, {0.0, 0.0, 1.0}};
    const double tc[3][3] = {{sc, 0.0, -sc * pd->cen[2]}, {0.0, sc, -sc * pd->cen[3]}, {0.0, 0.0, 1.0}};
    double m1[3][3], ef[3][3];
    bool finite = true;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m1[i][j] = (tc[0][i] * ec[0][j] + tc[1][i] * ec[1][j]) + tc[2][i] * ec[2][j];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            ef[i][j] = (m1[i][0] * tp[0][j] + m1[i][1] * tp[1][j]) + m1[i][2] * tp[2][j];
            finite = finite && isfinite(ef[i][j]);
        }
    if (!finite) {
        pd->failed = 1;
        write_empty_result(results + ch.pair, pd->n, 0);
        return;
    }
    // DecomposeEssential: U, V in SO(3); R1 = U W V^T, R2 = U W^T V^T, t = U col 2
    svd3(ef, u, sv, v);
    const double detv = v[0][0] * (v[1][1] * v[2][2] - v[1][2] * v[2][1]) -
                        v[0][1] * (v[1][0] * v[2][2] - v[1][2] * v[2][0]) +
                        v[0][2] * (v[1][0] * v[2][1] - v[1][1] * v[2][0]);
    if (detv < 0.0)
        for (int i = 0; i < 3; ++i) v[i][2] = -v[i][2];
    double r1[3][3], r2[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            // U W = [u2, -u1, u3], U W^T = [-u2, u1, u3]
            r1[i][j] = (u[i][1] * v[j][0] + -u[i][0] * v[j][1]) + u[i][2] * v[j][2];
            r2[i][j] = (-u[i][1] * v[j][0] + u[i][0] * v[j][1]) + u[i][2] * v[j][2];
        }
    for (int k = 0; k < 4; ++k) {
        const double(*R)[3] = k < 2 ? r1 : r2;
        const double sg = (k & 1) ? -1.0 : 1.0;
        for (int i = 0; i < 9; ++i) pd->cand[k][i] = R[i / 3][i % 3];
        for (int i = 0; i < 3; ++i) pd->cand[k][9 + i] = sg * u[i][2];
    }
}

// 4 warps per chunk: warp k scores candidate k on the chunk's 32 rows.
__global__ void __launch_bounds__(4 * TRI_ROWS)
k_tri_cheirality(TriParams P, const TriChunk* __restrict__ chunks, TriPairDev* pairs,
                 const double4_32a* __restrict__ rays, double4_32a* __restrict__ pts, int* ipart, unsigned* tickets,
                 uslam_tri_result* results) {
    const TriChunk ch = chunks[blockIdx.x];
    TriPairDev* pd = pairs + ch.pair;
    if (pd->failed) return;  // uniform over the pair: written by the previous phase
    const int cand = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = ch.begin + lane;
    bool in = false;
    if (r < ch.end) {
        double R[12];
#pragma unroll
        for (int i = 0; i < 12; ++i) R[i] = pd->cand[cand][i];
        const double4_32a q = rays[r];
        // rows: x_p p1.row(2) - p1.row(0), y_p p1.row(2) - p1.row(1),
        //       x_c p2.row(2) - p2.row(0), y_c p2.row(2) - p2.row(1); p1 = [I|0], p2 = [R|t]
        double a[4][4];
        a[0][0] = -1.0; a[0][1] = 0.0;  a[0][2] = q.x; a[0][3] = 0.0;
        a[1][0] = 0.0;  a[1][1] = -1.0; a[1][2] = q.y; a[1][3] = 0.0;
        a[2][0] = q.z * R[6] - R[0]; a[2][1] = q.z * R[7] - R[1]; a[2][2] = q.z * R[8] - R[2]; a[2][3] = q.z * R[11] - R[9];
        a[3][0] = q.w * R[6] - R[3]; a[3][1] = q.w * R[7] - R[4]; a[3][2] = q.w * R[8] - R[5]; a[3][3] = q.w * R[11] - R[10];
        double x[4];
        null4(a, x);
        double4_32a p = make_double4_32a(0.0, 0.0, 0.0, 0.0);  // w = 0: no point
        if (!(fabs(x[3]) < 1e-12)) {
            const double X = x[0] / x[3], Y = x[1] / x[3], Z = x[2] / x[3];
            if (isfinite(X) && isfinite(Y) && isfinite(Z)) {
                p = make_double4_32a(X, Y, Z, 1.0);
                const double zc = ((R[6] * X + R[7] * Y) + R[8] * Z) + R[11];
                in = Z > 0.0 && zc > 0.0;
            }
        }
        pts[static_cast<size_t>(cand) * P.total + r] = p;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) ipart[static_cast<size_t>(blockIdx.x) * 4 + cand] = __popc(bal);
    if (!last_chunk(tickets + ch.pair, pd->nchunks)) return;
    if (threadIdx.x != 0) return;
    int best = 0, best_count = 0;
    for (int k = 0; k < 4; ++k) {
        int s = 0;
        for (int c = 0; c < pd->nchunks; ++c) s += __ldcg(ipart + static_cast<size_t>(pd->first_chunk + c) * 4 + k);
        pd->in_front[k] = s;
        if (s > best_count) {
            best_count = s;
            best = k;
        }
    }
    pd->best = best;
    if (best_count == 0) {
        pd->failed = 1;
        write_empty_result(results + ch.pair, pd->n, 0);
    }
}

__global__ void __launch_bounds__(TRI_ROWS)
k_tri_landmarks(TriParams P, const TriChunk* __restrict__ chunks, TriPairDev* pairs,
                const double4_32a* __restrict__ px, const double4_32a* __restrict__ pts, double4_32a* __restrict__ lm,
                uint8_t* __restrict__ keep, double* part, int* ipart, unsigned* tickets,
                uslam_tri_result* results) {
    const TriChunk ch = chunks[blockIdx.x];
    TriPairDev* pd = pairs + ch.pair;
    if (pd->failed) return;
    const int lane = threadIdx.x;
    const int r = ch.begin + lane;
    const int best = pd->best;
    double R[12];
#pragma unroll
    for (int i = 0; i < 12; ++i) R[i] = pd->cand[best][i];
    double err = 0.0;
    bool ok = false;
    if (r < ch.end) {
        const double4_32a p = pts[static_cast<size_t>(best) * P.total + r];
        if (p.w != 0.0) {
            const double cx = ((R[0] * p.x + R[1] * p.y) + R[2] * p.z) + R[9];
            const double cy = ((R[3] * p.x + R[4] * p.y) + R[5] * p.z) + R[10];
            const double cz = ((R[6] * p.x + R[7] * p.y) + R[8] * p.z) + R[11];
            const bool depth_ok = !(p.z < P.min_depth || p.z > P.max_depth || cz < P.min_depth || cz > P.max_depth);
            double u0, v0, u1, v1;
            if (depth_ok && project_to_pixel(p.x, p.y, p.z, P, u0, v0) && project_to_pixel(cx, cy, cz, P, u1, v1)) {
                const double4_32a q = px[r];
                const double ex0 = u0 - q.x, ey0 = v0 - q.y, ex1 = u1 - q.z, ey1 = v1 - q.w;
                const double e = 0.5 * (sqrt(ex0 * ex0 + ey0 * ey0) + sqrt(ex1 * ex1 + ey1 * ey1));
                if (!(e > P.max_reproj)) {
                    ok = true;
                    err = e;
                    lm[r] = make_double4_32a(cx, cy, cz, e);
                }
            }
        }
        keep[r] = ok ? 1 : 0;
    }
    const double se = warp_sum(err);
    const int cnt = __popc(__ballot_sync(0xffffffffu, ok));
    if (lane == 0) {
        part[static_cast<size_t>(blockIdx.x) * TRI_PART] = se;
        ipart[static_cast<size_t>(blockIdx.x) * 4] = cnt;
    }
    if (!last_chunk(tickets + ch.pair, pd->nchunks)) return;
    if (lane != 0) return;
    double sum = 0.0;
    int count = 0;
    for (int c = 0; c < pd->nchunks; ++c) {
        sum += __ldcg(part + static_cast<size_t>(pd->first_chunk + c) * TRI_PART);
        count += __ldcg(ipart + static_cast<size_t>(pd->first_chunk + c) * 4);
    }
    uslam_tri_result* o = results + ch.pair;
    for (int i = 0; i < 9; ++i) o->rotation[i] = R[i];
    for (int i = 0; i < 3; ++i) o->translation[i] = R[9 + i];
    o->input_matches = pd->n;
    o->landmark_count = count;
    o->cheirality_passes = pd->in_front[best];
    o->pose_recovered = count > 0;
    o->mean_reprojection_error_px = count > 0 ? sum / static_cast<double>(count) : 0.0;
    // ComputeRotationAngle (map_helpers_lods.hpp:33-36)
    const double tr = fmin(fmax((R[0] + R[4]) + R[8], -1.0), 3.0);
    o->rotation_angle_rad = acos(fmin(fmax(0.5 * (tr - 1.0), -1.0), 1.0));
}

// CollectInliers' undistortion alone (uslam_pixel_to_normalised).
__global__ void k_tri_undistort(TriParams P, const double2* __restrict__ px, int n, double2* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double2 q = px[i];
        double x, y;
        pixel_to_normalised(q.x, q.y, P, x, y);
        out[i] = make_double2(x, y);
    }
}

TriParams make_params(const uslam_camera* cam) {
    TriParams P;
    std::memset(&P, 0, sizeof(P));
    P.fu = cam->fu;
    P.fv = cam->fv;
    P.cu = cam->cu;
    P.cv = cam->cv;
    P.k1 = cam->k1;
    P.k2 = cam->k2;
    P.p1 = cam->p1;
    P.p2 = cam->p2;
    return P;
}

// Grows the context's triangulation scratch to at least `need` bytes
// (the caller holds tri_mu).
cudaError_t tri_scratch(uslam_ctx* ctx, size_t need) {
    if (need <= ctx->tri_bytes) return cudaSuccess;
    if (ctx->tri_buf) cudaFree(ctx->tri_buf);
    ctx->tri_buf = nullptr;
    ctx->tri_bytes = 0;
    const cudaError_t e = cudaMalloc(&ctx->tri_buf, need);
    if (e == cudaSuccess) ctx->tri_bytes = need;
    return e;
}

}  // namespace

extern "C" {

uslam_status uslam_pixel_to_normalised(uslam_ctx* ctx, const uslam_camera* cam, int iterations, double tolerance,
                                       const double* px, int n, double* out) {
    if (!ctx || !cam || n < 0 || iterations < 0 || (n > 0 && (!px || !out)))
        return set_err(ctx ? &ctx->err : nullptr, USLAM_INVALID_ARG, "pixel_to_normalised: bad arguments");
    if (n == 0) return USLAM_OK;
    TriParams P = make_params(cam);
    P.iters = iterations;
    P.tol = tolerance;
    const size_t b = uslam_rt::round_up(sizeof(double2) * static_cast<size_t>(n), 256);
    cudaError_t e = cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->tri_mu);
    if (e == cudaSuccess) e = tri_scratch(ctx, 2 * b);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "pixel_to_normalised: scratch");
    double2* d_in = static_cast<double2*>(ctx->tri_buf);
    double2* d_out = reinterpret_cast<double2*>(static_cast<char*>(ctx->tri_buf) + b);
    e = cudaMemcpy(d_in, px, sizeof(double2) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int grid = std::min((n + 127) / 128, std::max(ctx->num_sms, 1) * 16);
        k_tri_undistort<<<grid, 128>>>(P, d_in, n, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, sizeof(double2) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "pixel_to_normalised");
    return USLAM_OK;
}

uslam_status uslam_triangulate(uslam_ctx* ctx, const uslam_camera* cam, const uslam_tri_opts* opts, int n_pairs,
                               const int* offsets, const double* px, uslam_tri_result* results, double* landmarks,
                               uint8_t* keep) {
    ErrText* err = ctx ? &ctx->err : nullptr;
    if (!ctx || !cam || n_pairs < 0 || (n_pairs > 0 && (!offsets || !results)))
        return set_err(err, USLAM_INVALID_ARG, "triangulate: bad arguments");
    uslam_tri_opts o;
    if (opts) {
        o = *opts;
    } else {
        uslam_tri_default_opts(&o);
    }
    if (o.min_inliers < 8 || o.undistort_iterations < 0 || !(o.max_reprojection_px >= 0.0) ||
        !(o.max_depth >= o.min_depth))
        return set_err(err, USLAM_INVALID_ARG, "triangulate: bad options (min_inliers >= 8 is required)");
    if (n_pairs == 0) return USLAM_OK;
    if (offsets[0] != 0) return set_err(err, USLAM_INVALID_ARG, "triangulate: offsets[0] must be 0");
    for (int p = 0; p < n_pairs; ++p)
        if (offsets[p + 1] < offsets[p]) return set_err(err, USLAM_INVALID_ARG, "triangulate: offsets decrease");
    const int total = offsets[n_pairs];
    if (total > 0 && !px) return set_err(err, USLAM_INVALID_ARG, "triangulate: px is NULL");

    // pairs below min_inliers get the reference's empty result on the host
    // (triangulate_cpu.cpp:365-374); the others are cut into chunks
    std::vector<TriPairDev> pairs(n_pairs);
    std::vector<TriChunk> chunks;
    int active = 0;
    for (int p = 0; p < n_pairs; ++p) {
        TriPairDev& d = pairs[p];
        std::memset(&d, 0, sizeof(d));
        d.begin = offsets[p];
        d.n = offsets[p + 1] - offsets[p];
        d.first_chunk = static_cast<int>(chunks.size());
        if (d.n < o.min_inliers) {
            d.failed = 1;
            continue;
        }
        ++active;
        for (int b = d.begin; b < d.begin + d.n; b += TRI_ROWS)
            chunks.push_back(TriChunk{p, b, std::min(b + TRI_ROWS, d.begin + d.n), 0});
        d.nchunks = static_cast<int>(chunks.size()) - d.first_chunk;
    }
    auto host_empty = [&](int p) {
        uslam_tri_result& r = results[p];
        std::memset(&r, 0, sizeof(r));
        r.rotation[0] = r.rotation[4] = r.rotation[8] = 1.0;
        r.input_matches = pairs[p].n;
    };
    if (landmarks) std::memset(landmarks, 0, sizeof(double) * 4 * static_cast<size_t>(total));
    if (keep) std::memset(keep, 0, static_cast<size_t>(total));
    if (active == 0) {
        for (int p = 0; p < n_pairs; ++p) host_empty(p);
        return USLAM_OK;
    }
    const int nch = static_cast<int>(chunks.size());

    using uslam_rt::round_up;
    const size_t b_pairs = round_up(sizeof(TriPairDev) * n_pairs, 256);
    const size_t b_chunks = round_up(sizeof(TriChunk) * nch, 256);
    const size_t b_tick = round_up(sizeof(unsigned) * n_pairs, 256);
    const size_t b_part = round_up(sizeof(double) * TRI_PART * nch, 256);
    const size_t b_ipart = round_up(sizeof(int) * 4 * nch, 256);
    const size_t b_rows = round_up(sizeof(double4_32a) * total, 256);
    const size_t b_keep = round_up(static_cast<size_t>(total), 256);
    const size_t b_res = round_up(sizeof(uslam_tri_result) * n_pairs, 256);
    // px, rays, 4 candidate point sets, landmarks
    const size_t need = b_pairs + b_chunks + b_tick + b_part + b_ipart + 7 * b_rows + b_keep + b_res;

    cudaError_t e = cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->tri_mu);
    if (e == cudaSuccess) e = tri_scratch(ctx, need);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "triangulate: scratch");
    char* base = static_cast<char*>(ctx->tri_buf);
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        char* p = base + off;
        off += bytes;
        return p;
    };
    TriPairDev* d_pairs = reinterpret_cast<TriPairDev*>(carve(b_pairs));
    TriChunk* d_chunks = reinterpret_cast<TriChunk*>(carve(b_chunks));
    unsigned* d_tick = reinterpret_cast<unsigned*>(carve(b_tick));
    double* d_part = reinterpret_cast<double*>(carve(b_part));
    int* d_ipart = reinterpret_cast<int*>(carve(b_ipart));
    double4_32a* d_px = reinterpret_cast<double4_32a*>(carve(b_rows));
    double4_32a* d_rays = reinterpret_cast<double4_32a*>(carve(b_rows));
    double4_32a* d_pts = reinterpret_cast<double4_32a*>(carve(4 * b_rows));
    double4_32a* d_lm = reinterpret_cast<double4_32a*>(carve(b_rows));
    uint8_t* d_keep = reinterpret_cast<uint8_t*>(carve(b_keep));
    uslam_tri_result* d_res = reinterpret_cast<uslam_tri_result*>(carve(b_res));

    TriParams P = make_params(cam);
    P.max_reproj = o.max_reprojection_px;
    P.min_depth = o.min_depth;
    P.max_depth = o.max_depth;
    P.tol = o.undistort_tolerance;
    P.iters = o.undistort_iterations;
    P.total = total;

    e = cudaMemcpy(d_pairs, pairs.data(), sizeof(TriPairDev) * n_pairs, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_chunks, chunks.data(), sizeof(TriChunk) * nch, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_px, px, sizeof(double4_32a) * total, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_tick, 0, sizeof(unsigned) * n_pairs);
    if (e == cudaSuccess) e = cudaMemset(d_lm, 0, sizeof(double4_32a) * total);
    if (e == cudaSuccess) e = cudaMemset(d_keep, 0, static_cast<size_t>(total));
    if (e == cudaSuccess) {
        k_tri_rays<<<nch, TRI_ROWS>>>(P, d_chunks, d_pairs, d_px, d_rays, d_part, d_tick);
        k_tri_spread<<<nch, TRI_ROWS>>>(d_chunks, d_pairs, d_rays, d_part, d_tick);
        k_tri_gram<<<nch, TRI_ROWS>>>(d_chunks, d_pairs, d_rays, d_part, d_tick, d_res);
        k_tri_cheirality<<<nch, 4 * TRI_ROWS>>>(P, d_chunks, d_pairs, d_rays, d_pts, d_ipart, d_tick, d_res);
        k_tri_landmarks<<<nch, TRI_ROWS>>>(P, d_chunks, d_pairs, d_px, d_pts, d_lm, d_keep, d_part, d_ipart, d_tick,
                                           d_res);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(results, d_res, sizeof(uslam_tri_result) * n_pairs, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && landmarks)
        e = cudaMemcpy(landmarks, d_lm, sizeof(double4_32a) * total, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && keep) e = cudaMemcpy(keep, d_keep, static_cast<size_t>(total), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "triangulate");
    for (int p = 0; p < n_pairs; ++p)
        if (pairs[p].n < o.min_inliers) host_empty(p);
    return USLAM_OK;
}

void uslam_tri_default_opts(uslam_tri_opts* o) {
    if (!o) return;
    // TriangulateCPU::Opts (wslam/src/pose_estimate_cpu/triangulate_cpu.hpp:30-54)
    o->max_reprojection_px = 4.0;
    o->min_depth = 1e-3;
    o->max_depth = 1e3;
    o->undistort_tolerance = 1e-9;
    o->min_inliers = 8;
    o->undistort_iterations = 20;
}

}  // extern "C"
