// Exact geometry over a triangle mesh for every point of a batch: the signed
// solid angle the mesh subtends (van Oosterom; src/mbem/geometry.py:8-57,
// read as the region classifier RegionModel.point_in_region,
// src/mbem/model/core.py:994-1025) and the distance to the nearest triangle
// with its index (src/mbem/geometry.py:60-105).
//
// One thread an observer, 128 observers a CTA, the triangles staged through
// shared memory 128 at a time as 128-byte records that a prepare kernel
// builds once per mesh. A (point, triangle) pair farther than GEOM_NEAR_K
// circumradii from the centroid runs in FP32 on coordinates split into
// hi + lo floats, so a - p is formed to ~1e-7 of |a - p| whatever the
// coordinates' magnitude, with the triple product taken against the
// triangle's own 2A n (a . (b x c) = a . ((b - a) x (c - a))); nearer pairs
// run the reference's FP64 arithmetic. The FP64 rate of this part is about a
// sixtieth of its FP32 rate, and almost every pair of a volume grid is far.
//
// Solid angle: the FP32 far terms of a tile of 128 triangles in a
// compensated (Kahan) FP32 sum, added to an FP64 total once a tile.
// Error analysis: each far term carries ~1e-7 x 2A/D^2 from a - p and 2 ulp
// from atan2f; over a closed surface the sum is within ~1e-6 steradian of
// the FP64 sum (the classifier's band is 1e-6 x 4 pi = 1.26e-5).
//
// Distance: a first FP32 sweep finds the smallest distance d32; a second
// sweep evaluates in FP64 (the reference's Voronoi-region projection) every
// triangle whose FP32 distance is within 1e-4 (d32 + longest edge) of it,
// a margin a hundred times the FP32 error, and keeps the smallest (ties:
// nearer centroid, then lower index). The reference searches the 32
// triangles with the nearest centroids (cKDTree); this searches all of them,
// so it returns the same triangle whenever that search contained the
// nearest one.
#include <math.h>

#include "common.cuh"

namespace mbem {

namespace {

constexpr int GEOM_THREADS = 128;     // observers a CTA and records a tile
constexpr int GEOM_REC = 32;          // floats a record
// FP64 inside this many circumradii: beyond, every vertex is at least one
// circumradius away and the triangle subtends under 60 degrees, so the
// van Oosterom denominator is a sum of positive terms (no cancellation)
constexpr float GEOM_NEAR_K = 2.0f;

// record: [0..8] vertex hi (a b c), [9..17] vertex lo, [18..20] b - a,
// [21..23] c - a, [24..26] (b - a) x (c - a), [27..29] centroid (hi),
// [30] (GEOM_NEAR_K x circumradius)^2, [31] unused
__global__ void __launch_bounds__(128) geom_prep_kernel(const double* __restrict__ tv, int64_t nt,
                                                        float* __restrict__ rec) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double v[9];
#pragma unroll
    for (int k = 0; k < 9; k++) v[k] = tv[t * 9 + k];
    float* r = rec + t * GEOM_REC;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const float hi = (float)v[k];
        r[k] = hi;
        r[9 + k] = (float)(v[k] - (double)hi);
    }
    double e1[3], e2[3], cen[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        e1[k] = v[3 + k] - v[k];
        e2[k] = v[6 + k] - v[k];
        cen[k] = (v[k] + v[3 + k] + v[6 + k]) / 3.0;
        r[18 + k] = (float)e1[k];
        r[21 + k] = (float)e2[k];
        r[27 + k] = (float)cen[k];
    }
    r[24] = (float)(e1[1] * e2[2] - e1[2] * e2[1]);
    r[25] = (float)(e1[2] * e2[0] - e1[0] * e2[2]);
    r[26] = (float)(e1[0] * e2[1] - e1[1] * e2[0]);
    double rmax2 = 0.0;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const double dx = v[3 * q] - cen[0], dy = v[3 * q + 1] - cen[1], dz = v[3 * q + 2] - cen[2];
        rmax2 = fmax(rmax2, dx * dx + dy * dy + dz * dz);
    }
    r[30] = (float)((double)GEOM_NEAR_K * (double)GEOM_NEAR_K * rmax2);
    r[31] = 0.0f;
}

__device__ __forceinline__ void stage_tile(const float* __restrict__ rec, int64_t t0, int64_t nt, float* s) {
    // GEOM_THREADS records of 8 float4s, one float4 a thread per step
    const float4* src = reinterpret_cast<const float4*>(rec + t0 * GEOM_REC);
    float4* dst = reinterpret_cast<float4*>(s);
    const int64_t n4 = lmin(GEOM_THREADS, nt - t0) * (GEOM_REC / 4);
    for (int64_t q = threadIdx.x; q < n4; q += GEOM_THREADS) dst[q] = src[q];
}

// (vertex - point) from the hi/lo split: exact hi difference rounding plus
// the lo difference, ~1e-7 of the result
__device__ __forceinline__ float rel(float vhi, float vlo, float phi, float plo) { return (vhi - phi) + (vlo - plo); }

// the reference's van Oosterom term in FP64 (src/mbem/geometry.py:24-46)
__device__ double omega_fp64(const double* __restrict__ tv, int64_t t, double px, double py, double pz) {
    const double* v = tv + t * 9;
    const double ax = v[0] - px, ay = v[1] - py, az = v[2] - pz;
    const double bx = v[3] - px, by = v[4] - py, bz = v[5] - pz;
    const double cx = v[6] - px, cy = v[7] - py, cz = v[8] - pz;
    const double ra = sqrt(ax * ax + ay * ay + az * az);
    const double rb = sqrt(bx * bx + by * by + bz * bz);
    const double rc = sqrt(cx * cx + cy * cy + cz * cz);
    const double numer = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
    const double denom = ra * rb * rc + rc * (ax * bx + ay * by + az * bz) + ra * (bx * cx + by * cy + bz * cz) +
                         rb * (ax * cx + ay * cy + az * cz);
    return 2.0 * atan2(numer, denom);
}

__global__ void __launch_bounds__(GEOM_THREADS) solid_angle_kernel(const float* __restrict__ rec,
                                                                   const double* __restrict__ tv, int64_t nt,
                                                                   const double* __restrict__ pts, int64_t n,
                                                                   double weight, int accumulate,
                                                                   double* __restrict__ total) {
    __shared__ __align__(16) float s[GEOM_THREADS * GEOM_REC];
    const int64_t i = (int64_t)blockIdx.x * GEOM_THREADS + threadIdx.x;
    const bool live = i < n;
    double px = 0.0, py = 0.0, pz = 0.0;
    if (live) {
        px = pts[3 * i];
        py = pts[3 * i + 1];
        pz = pts[3 * i + 2];
    }
    const float phx = (float)px, phy = (float)py, phz = (float)pz;
    const float plx = (float)(px - (double)phx), ply = (float)(py - (double)phy), plz = (float)(pz - (double)phz);
    double sum = 0.0;
    for (int64_t t0 = 0; t0 < nt; t0 += GEOM_THREADS) {
        __syncthreads();
        stage_tile(rec, t0, nt, s);
        __syncthreads();
        const int cnt = (int)lmin(GEOM_THREADS, nt - t0);
        if (!live) continue;
        float part = 0.0f, comp = 0.0f;      // Kahan sum of the tile's far terms
        for (int j0 = 0; j0 < cnt; j0 += 4) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int j = j0 + u;
                if (j >= cnt) break;
                const float* r = s + j * GEOM_REC;
                const float dcx = r[27] - phx, dcy = r[28] - phy, dcz = r[29] - phz;
                if (dcx * dcx + dcy * dcy + dcz * dcz <= r[30]) {
                    sum += omega_fp64(tv, t0 + j, px, py, pz);
                    continue;
                }
                const float ax = rel(r[0], r[9], phx, plx), ay = rel(r[1], r[10], phy, ply),
                            az = rel(r[2], r[11], phz, plz);
                const float bx = rel(r[3], r[12], phx, plx), by = rel(r[4], r[13], phy, ply),
                            bz = rel(r[5], r[14], phz, plz);
                const float cx = rel(r[6], r[15], phx, plx), cy = rel(r[7], r[16], phy, ply),
                            cz = rel(r[8], r[17], phz, plz);
                const float ra2 = ax * ax + ay * ay + az * az, rb2 = bx * bx + by * by + bz * bz,
                            rc2 = cx * cx + cy * cy + cz * cz;
                const float ra = ra2 * rsqrtf(ra2), rb = rb2 * rsqrtf(rb2), rc = rc2 * rsqrtf(rc2);
                const float numer = ax * r[24] + ay * r[25] + az * r[26];
                const float denom = ra * rb * rc + rc * (ax * bx + ay * by + az * bz) +
                                    ra * (bx * cx + by * cy + bz * cz) + rb * (ax * cx + ay * cy + az * cz);
                const float y = 2.0f * atan2f(numer, denom) - comp;
                const float t = part + y;
                comp = (t - part) - y;
                part = t;
            }
        }
        sum += (double)part - (double)comp;
    }
    if (live) total[i] = (accumulate ? total[i] : 0.0) + weight * sum;
}

// squared FP32 distance from the point to the record's triangle (the
// Voronoi-region closest point, as in the FP64 form below)
__device__ __forceinline__ float dist2_f32(const float* r, float phx, float phy, float phz, float plx, float ply,
                                           float plz) {
    // ap = p - a etc.
    const float apx = -rel(r[0], r[9], phx, plx), apy = -rel(r[1], r[10], phy, ply), apz = -rel(r[2], r[11], phz, plz);
    const float bpx = -rel(r[3], r[12], phx, plx), bpy = -rel(r[4], r[13], phy, ply), bpz = -rel(r[5], r[14], phz, plz);
    const float cpx = -rel(r[6], r[15], phx, plx), cpy = -rel(r[7], r[16], phy, ply), cpz = -rel(r[8], r[17], phz, plz);
    const float abx = r[18], aby = r[19], abz = r[20], acx = r[21], acy = r[22], acz = r[23];
    const float d1 = abx * apx + aby * apy + abz * apz, d2 = acx * apx + acy * apy + acz * apz;
    const float d3 = abx * bpx + aby * bpy + abz * bpz, d4 = acx * bpx + acy * bpy + acz * bpz;
    const float d5 = abx * cpx + aby * cpy + abz * cpz, d6 = acx * cpx + acy * cpy + acz * cpz;
    float qx, qy, qz;   // q - a
    if (d6 >= 0.0f && d5 <= d6) {
        qx = acx; qy = acy; qz = acz;
    } else if (d3 >= 0.0f && d4 <= d3) {
        qx = abx; qy = aby; qz = abz;
    } else if (d1 <= 0.0f && d2 <= 0.0f) {
        qx = qy = qz = 0.0f;
    } else {
        const float va = d3 * d6 - d5 * d4, vb = d5 * d2 - d1 * d6, vc = d1 * d4 - d3 * d2;
        if (va <= 0.0f && d4 >= d3 && d5 >= d6) {
            const float e = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            qx = abx + (acx - abx) * e; qy = aby + (acy - aby) * e; qz = abz + (acz - abz) * e;
        } else if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
            const float e = d2 / (d2 - d6);
            qx = acx * e; qy = acy * e; qz = acz * e;
        } else if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
            const float e = d1 / (d1 - d3);
            qx = abx * e; qy = aby * e; qz = abz * e;
        } else {
            const float sv = va + vb + vc;
            const float wb = vb / sv, wc = vc / sv;
            qx = abx * wb + acx * wc; qy = aby * wb + acy * wc; qz = abz * wb + acz * wc;
        }
    }
    const float dx = apx - qx, dy = apy - qy, dz = apz - qz;
    return dx * dx + dy * dy + dz * dz;
}

// the reference's exact distance in FP64 (src/mbem/geometry.py:60-87): the
// plane projection replaced by the last Voronoi region whose test holds, in
// the order interior, edge ab, edge ac, edge bc, vertex a, vertex b, vertex c
__device__ double dist_fp64(const double* __restrict__ tv, int64_t t, double px, double py, double pz) {
    const double* v = tv + t * 9;
    const double a[3] = {v[0], v[1], v[2]}, b[3] = {v[3], v[4], v[5]}, c[3] = {v[6], v[7], v[8]};
    const double p[3] = {px, py, pz};
    double ab[3], ac[3], ap[3], bp[3], cp[3];
    for (int k = 0; k < 3; k++) {
        ab[k] = b[k] - a[k];
        ac[k] = c[k] - a[k];
        ap[k] = p[k] - a[k];
        bp[k] = p[k] - b[k];
        cp[k] = p[k] - c[k];
    }
    auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    const double d1 = dot(ab, ap), d2 = dot(ac, ap), d3 = dot(ab, bp), d4 = dot(ac, bp), d5 = dot(ab, cp),
                 d6 = dot(ac, cp);
    const double va = d3 * d6 - d5 * d4, vb = d5 * d2 - d1 * d6, vc = d1 * d4 - d3 * d2;
    double q[3];
    if (d6 >= 0.0 && d5 <= d6) {
        for (int k = 0; k < 3; k++) q[k] = c[k];
    } else if (d3 >= 0.0 && d4 <= d3) {
        for (int k = 0; k < 3; k++) q[k] = b[k];
    } else if (d1 <= 0.0 && d2 <= 0.0) {
        for (int k = 0; k < 3; k++) q[k] = a[k];
    } else if (va <= 0.0 && d4 >= d3 && d5 >= d6) {
        const double e = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        for (int k = 0; k < 3; k++) q[k] = b[k] + (c[k] - b[k]) * e;
    } else if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        const double e = d2 / (d2 - d6);
        for (int k = 0; k < 3; k++) q[k] = a[k] + ac[k] * e;
    } else if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        const double e = d1 / (d1 - d3);
        for (int k = 0; k < 3; k++) q[k] = a[k] + ab[k] * e;
    } else {
        const double s = va + vb + vc;
        for (int k = 0; k < 3; k++) q[k] = a[k] + ab[k] * (vb / s) + ac[k] * (vc / s);
    }
    const double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

__global__ void __launch_bounds__(GEOM_THREADS) mesh_distance_kernel(const float* __restrict__ rec,
                                                                     const double* __restrict__ tv, int64_t nt,
                                                                     const double* __restrict__ pts, int64_t n,
                                                                     float max_edge, double* __restrict__ dist,
                                                                     int64_t* __restrict__ idx) {
    __shared__ __align__(16) float s[GEOM_THREADS * GEOM_REC];
    const int64_t i = (int64_t)blockIdx.x * GEOM_THREADS + threadIdx.x;
    const bool live = i < n;
    double px = 0.0, py = 0.0, pz = 0.0;
    if (live) {
        px = pts[3 * i];
        py = pts[3 * i + 1];
        pz = pts[3 * i + 2];
    }
    const float phx = (float)px, phy = (float)py, phz = (float)pz;
    const float plx = (float)(px - (double)phx), ply = (float)(py - (double)phy), plz = (float)(pz - (double)phz);
    // sweep 1: the smallest FP32 distance
    float best2 = INFINITY;
    for (int64_t t0 = 0; t0 < nt; t0 += GEOM_THREADS) {
        __syncthreads();
        stage_tile(rec, t0, nt, s);
        __syncthreads();
        const int cnt = (int)lmin(GEOM_THREADS, nt - t0);
        if (!live) continue;
        for (int j = 0; j < cnt; j++) best2 = fminf(best2, dist2_f32(s + j * GEOM_REC, phx, phy, phz, plx, ply, plz));
    }
    const float d32 = sqrtf(best2);
    const float thr = d32 + 1e-4f * (d32 + max_edge);
    const float thr2 = thr * thr;
    // sweep 2: FP64 on the candidates within the margin
    double bd = INFINITY, bc = INFINITY;
    int64_t bi = -1;
    for (int64_t t0 = 0; t0 < nt; t0 += GEOM_THREADS) {
        __syncthreads();
        stage_tile(rec, t0, nt, s);
        __syncthreads();
        const int cnt = (int)lmin(GEOM_THREADS, nt - t0);
        if (!live) continue;
        for (int j = 0; j < cnt; j++) {
            const float* r = s + j * GEOM_REC;
            if (!(dist2_f32(r, phx, phy, phz, plx, ply, plz) <= thr2)) continue;
            const int64_t t = t0 + j;
            const double d = dist_fp64(tv, t, px, py, pz);
            if (d > bd) continue;
            const double* v = tv + t * 9;
            const double cx = (v[0] + v[3] + v[6]) / 3.0 - px, cy = (v[1] + v[4] + v[7]) / 3.0 - py,
                         cz = (v[2] + v[5] + v[8]) / 3.0 - pz;
            const double c2 = cx * cx + cy * cy + cz * cz;
            if (d < bd || c2 < bc) {
                bd = d;
                bc = c2;
                bi = t;
            }
        }
    }
    if (live) {
        dist[i] = bd;
        idx[i] = bi;
    }
}

}  // namespace

}  // namespace mbem

using namespace mbem;

extern "C" {

size_t mbem_geom_record_bytes(int64_t n_tri) { return (size_t)(n_tri > 0 ? n_tri : 0) * GEOM_REC * sizeof(float); }

int mbem_geom_prepare(const double* tri_verts, int64_t n_tri, float* records, void* stream) {
    MBEM_REQUIRE(n_tri >= 0, MBEM_ERR_ARG, "bad triangle count");
    MBEM_REQUIRE(n_tri == 0 || (tri_verts && records), MBEM_ERR_ARG, "NULL mesh arrays");
    MBEM_REQUIRE(((uintptr_t)records & 15) == 0, MBEM_ERR_ARG, "records must be 16-byte aligned");
    if (n_tri == 0) return MBEM_OK;
    geom_prep_kernel<<<(unsigned)ceil_div(n_tri, 128), 128, 0, (cudaStream_t)stream>>>(tri_verts, n_tri, records);
    return launch_status("geom_prep_kernel");
}

int mbem_solid_angle_sum(const float* records, const double* tri_verts, int64_t n_tri, const double* points,
                         int64_t n_pts, double weight, int accumulate, double* total, void* stream) {
    MBEM_REQUIRE(n_tri >= 0 && n_pts >= 0, MBEM_ERR_ARG, "bad sizes");
    MBEM_REQUIRE(n_pts == 0 || (points && total), MBEM_ERR_ARG, "NULL point arrays");
    MBEM_REQUIRE(n_tri == 0 || (tri_verts && records), MBEM_ERR_ARG, "NULL mesh arrays");
    MBEM_REQUIRE(((uintptr_t)records & 15) == 0, MBEM_ERR_ARG, "records must be 16-byte aligned");
    if (n_pts == 0) return MBEM_OK;
    MBEM_REQUIRE(ceil_div(n_pts, GEOM_THREADS) < (int64_t)INT32_MAX, MBEM_ERR_SIZE, "too many points");
    solid_angle_kernel<<<(unsigned)ceil_div(n_pts, GEOM_THREADS), GEOM_THREADS, 0, (cudaStream_t)stream>>>(
        records, tri_verts, n_tri, points, n_pts, weight, accumulate, total);
    return launch_status("solid_angle_kernel");
}

int mbem_mesh_distance(const float* records, const double* tri_verts, int64_t n_tri, const double* points,
                       int64_t n_pts, double max_edge, double* dist, int64_t* idx, void* stream) {
    MBEM_REQUIRE(n_tri >= 1, MBEM_ERR_ARG, "the distance to a mesh needs at least one triangle");
    MBEM_REQUIRE(n_pts >= 0 && max_edge >= 0.0, MBEM_ERR_ARG, "bad sizes");
    MBEM_REQUIRE(tri_verts && records && (n_pts == 0 || (points && dist && idx)), MBEM_ERR_ARG, "NULL arrays");
    MBEM_REQUIRE(((uintptr_t)records & 15) == 0, MBEM_ERR_ARG, "records must be 16-byte aligned");
    if (n_pts == 0) return MBEM_OK;
    MBEM_REQUIRE(ceil_div(n_pts, GEOM_THREADS) < (int64_t)INT32_MAX, MBEM_ERR_SIZE, "too many points");
    mesh_distance_kernel<<<(unsigned)ceil_div(n_pts, GEOM_THREADS), GEOM_THREADS, 0, (cudaStream_t)stream>>>(
        records, tri_verts, n_tri, points, n_pts, (float)max_edge, dist, idx);
    return launch_status("mesh_distance_kernel");
}

}  // extern "C"
