// fxe_voronoi.cu — contact candidates, Voronoi contact surfaces and complementarity scoring.
//
// Kernels (one launch each per batch):
//   contacts_kernel  one warp per (pose, ligand atom): the 27-cell scan of get_contlist4
//                    (LIB/Vcontacts.cpp:1725-1839) over the receptor's cell list and the pose's
//                    ligand atoms, in the reference's candidate order, plus the atom's share of
//                    the clash pre-filter (LIB/Vcontacts.cpp:36-51).
//   voronoi_kernel   one warp per (pose, ligand atom): the extended-radical-plane polyhedron
//                    (voronoi_poly2, LIB/Vcontacts.cpp:147-490), its faces (order_faces,
//                    :699-831) and their spherical areas (calc_areas, :838-1044), FP32.
//   score_kernel     one warp per pose: replays the order-dependent bookkeeping of calc_region /
//                    save_areas (which contacts an atom keeps depends on the atoms processed
//                    before it), recomputing an atom with its reduced candidate list whenever a
//                    plane the reference would drop reaches that atom's sphere, then walks the
//                    kept contacts as vcfunction does (LIB/vcfunction.cpp:14-574).
//
// Every ligand atom's polyhedron is computed independently with its full candidate list. In
// exact arithmetic a plane the reference drops (an earlier atom that recorded no contact with
// this one) bounds no part of this atom's sphere, so the areas agree; score_kernel checks that
// per atom and recomputes the few atoms where it does not hold.
#include <cfloat>
#include <climits>

#include "fxe_common.cuh"

namespace fxe {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint8_t kNone = 255;
constexpr int kVorWarps = 4;

// ------------------------------------------------------------------------------------------
// per-warp workspace of one polyhedron
// ------------------------------------------------------------------------------------------
struct VorShared {
    float4 pl[kMaxPlanes];          // plane A.x + D = 0 (A unit normal, D = -plane distance)
    float area[kMaxCand];
    int cidx[kMaxCand];             // Calc index of each candidate
    float4 vx[kMaxVerts];           // vertex x, y, z, distance to the atom centre
    uchar4 vp[kMaxVerts];           // the vertex's planes (kNone = sphere)
    union {
        struct {
            float4 ev[kMaxEdges];   // edge direction
            uchar4 ep[kMaxEdges];   // plane0, plane1, start plane, end plane
            uchar2 es[kMaxEdges];   // start vertex, end vertex
        } e;
        struct {
            uint8_t pt[kMaxFacePts];
            float cosv[kMaxFacePts];
        } f;
    } u;
    uint16_t foff[kMaxCand + 1];
    uint8_t fnp[kMaxCand];
    uint8_t flag[kMaxPlanes];
    int eng[4];
    int epi;
    int nv;
};

__device__ __forceinline__ void warp_argmin(float& v, int& i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float v2 = __shfl_xor_sync(kFull, v, o);
        const int i2 = __shfl_xor_sync(kFull, i, o);
        if (v2 < v || (v2 == v && i2 < i)) {
            v = v2;
            i = i2;
        }
    }
}

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int* total) {
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    *total = __shfl_sync(kFull, x, 31);
    return x - v;
}

__device__ __forceinline__ float dot3(const float4& a, float x, float y, float z) {
    return a.x * x + a.y * y + a.z * z;
}

// solve_3x3 (LIB/Vcontacts.cpp:1384-1414) in FP32.
__device__ bool solve3(const float4& e0, const float4& e1, const float4& e2, float* pt) {
    const float c00 = e1.y * e2.z - e2.y * e1.z;
    const float c01 = -e1.x * e2.z + e2.x * e1.z;
    const float c02 = e1.x * e2.y - e2.x * e1.y;
    const float c10 = -e0.y * e2.z + e2.y * e0.z;
    const float c11 = e0.x * e2.z - e2.x * e0.z;
    const float c12 = -e0.x * e2.y + e2.x * e0.y;
    const float c20 = e0.y * e1.z - e1.y * e0.z;
    const float c21 = -e0.x * e1.z + e1.x * e0.z;
    const float c22 = e0.x * e1.y - e1.x * e0.y;
    const float det = e0.x * c00 + e0.y * c01 + e0.z * c02;
    if (det == 0.0f) return false;
    pt[0] = -(e0.w * c00 + e1.w * c10 + e2.w * c20) / det;
    pt[1] = -(e0.w * c01 + e1.w * c11 + e2.w * c21) / det;
    pt[2] = -(e0.w * c02 + e1.w * c12 + e2.w * c22) / det;
    return true;
}

// solve_2xS (LIB/Vcontacts.cpp:1427-1476) in FP32.
__device__ bool solve2s(const float4& a, const float4& b, float rado, float* p0, float* p1) {
    const float e2x = a.y * b.z - a.z * b.y;
    const float e2y = a.z * b.x - a.x * b.z;
    const float e2z = a.x * b.y - a.y * b.x;
    const float c00 = b.y * e2z - e2y * b.z;
    const float c01 = -b.x * e2z + e2x * b.z;
    const float c02 = b.x * e2y - e2x * b.y;
    const float c10 = -a.y * e2z + e2y * a.z;
    const float c11 = a.x * e2z - e2x * a.z;
    const float c12 = -a.x * e2y + e2x * a.y;
    const float det = e2x * e2x + e2y * e2y + e2z * e2z;
    if (det == 0.0f) return false;
    const float ax = -(a.w * c00 + b.w * c10) / det;
    const float ay = -(a.w * c01 + b.w * c11) / det;
    const float az = -(a.w * c02 + b.w * c12) / det;
    float t = (rado * rado - ax * ax - ay * ay - az * az) / det;
    if (t < 0.0f) return false;
    t = sqrtf(t);
    p0[0] = ax + t * e2x; p0[1] = ay + t * e2y; p0[2] = az + t * e2z;
    p1[0] = ax - t * e2x; p1[1] = ay - t * e2y; p1[2] = az - t * e2z;
    return true;
}

__device__ __forceinline__ float cos_pqr(const float4& p, const float4& q, const float4& r) {
    const float ax = p.x - q.x, ay = p.y - q.y, az = p.z - q.z;
    const float bx = r.x - q.x, by = r.y - q.y, bz = r.z - q.z;
    return (ax * bx + ay * by + az * bz) / sqrtf((ax * ax + ay * ay + az * az) * (bx * bx + by * by + bz * bz));
}

// spherical_arc (LIB/Vcontacts.cpp:1518-1557): cap segment between B and C about the contact
// centre Ao, minus the spherical triangle Ao-B-C.
__device__ float sph_arc(const float4& ao, const float4& b, const float4& c, float rado) {
    const float cosAOB = (ao.x * b.x + ao.y * b.y + ao.z * b.z) / (ao.w * b.w);
    const float cosBOC = (b.x * c.x + b.y * c.y + b.z * c.z) / (b.w * c.w);
    const float s = sqrtf((1.0f + cosBOC) / 8.0f);
    const float U = (1.0f + cosAOB) * s;
    const float V = (1.0f - cosAOB) * s;
    const float W = sqrtf((1.0f - cosAOB) * (1.0f + cosAOB) * (1.0f - cosBOC) / 8.0f);
    const float tS = (1.0f - U + V + W + W) / (1.0f + U - V - W - W);
    const float tSB = (1.0f - U - V) / (1.0f + U + V);
    const float tSA = (1.0f - U + V - W - W) / (1.0f + U - V + W + W);
    float tanprod = 0.0f;
    if (tS * tSA > 0.0f) tanprod = sqrtf(tSB * tSB * tS * tSA);
    const float cosBAC = cos_pqr(b, ao, c);
    float angBAC;
    if (cosBAC > 1.0f) angBAC = 0.0f;
    else if (cosBAC < -1.0f) angBAC = (float)kPi;
    else angBAC = acosf(cosBAC);
    return rado * (angBAC * (rado - ao.w) - 4.0f * rado * atanf(sqrtf(tanprod)));
}

__device__ __forceinline__ float4 centre_of(const float4& pl) {
    return make_float4(-pl.x * pl.w, -pl.y * pl.w, -pl.z * pl.w, fabsf(pl.w));
}

// test_point (LIB/Vcontacts.cpp:1357-1372): true unless x lies behind a contact plane.
__device__ bool inside_all(const VorShared& sh, int NC, int skip, float x, float y, float z) {
    for (int cp = 0; cp < NC; ++cp) {
        if (cp == skip || sh.flag[cp] == 0) continue;
        if (dot3(sh.pl[cp], x, y, z) + sh.pl[cp].w > 0.0f) return false;
    }
    return true;
}

__device__ void add_edge(VorShared& sh, int en, int p0, int p1, int tp, int sp) {
    const float4 a = sh.pl[p0], b = sh.pl[p1];
    float vx = a.y * b.z - a.z * b.y;
    float vy = a.z * b.x - a.x * b.z;
    float vz = a.x * b.y - a.y * b.x;
    const float4 s = sh.vx[sp];
    const float4 t = sh.pl[tp];
    const float tv = t.x * (s.x + vx) + t.y * (s.y + vy) + t.z * (s.z + vz) + t.w;
    if (tv > 0.0f) { vx = -vx; vy = -vy; vz = -vz; }
    sh.u.e.ev[en] = make_float4(vx, vy, vz, 0.0f);
    sh.u.e.ep[en] = make_uchar4((uint8_t)p0, (uint8_t)p1, (uint8_t)tp, kNone);
    sh.u.e.es[en] = make_uchar2((uint8_t)sp, kNone);
}

// One extended-radical-plane polyhedron and its contact areas. sh.pl/flag/cidx hold the
// planes of the NC candidates (excluded slots carry a plane that never binds). Returns
// kAtomOk, kAtomHullFail (the walk reached 200 edges) or kAtomCapacity.
__device__ int voronoi_warp(VorShared& sh, int NC, float rado, int lane, int* no_partner) {
    const float rr = rado * rado;
    // bounding planes
    if (lane < 4) {
        const float bx[4] = {0.707f, 0.707f, -0.707f, -0.707f};
        const float by[4] = {1.0f, -1.0f, 0.0f, 0.0f};
        const float bz[4] = {0.0f, 0.0f, 1.0f, -1.0f};
        sh.pl[NC + lane] = make_float4(bx[lane], by[lane], bz[lane], -10.0f);
        sh.flag[NC + lane] = 0;
    }
    for (int c = lane; c < NC; c += 32) sh.area[c] = 0.0f;
    __syncwarp();

    // ---- first vertex (get_firstvert without a seed, LIB/Vcontacts.cpp:532-590) ----
    float bv = 9.9e9f;
    int bi = INT_MAX;
    for (int c = lane; c < NC; c += 32) {
        const float d = fabsf(sh.pl[c].w);
        if (d < bv) { bv = d; bi = c; }
    }
    warp_argmin(bv, bi);
    const int pA0 = bi;
    if (pA0 == INT_MAX) return kAtomCapacity;
    const float4 A = sh.pl[pA0];
    bv = 9.9e9f;
    bi = INT_MAX;
    for (int c = lane; c < NC + 4; c += 32) {
        if (c == pA0) continue;
        const float4 C = sh.pl[c];
        const float4 v = make_float4(A.y * C.z - A.z * C.y, A.z * C.x - A.x * C.z, A.x * C.y - A.y * C.x, 0.0f);
        float t[3];
        if (solve3(A, C, v, t)) {
            const float d = sqrtf(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
            if (d < bv) { bv = d; bi = c; }
        }
    }
    warp_argmin(bv, bi);
    const int pB0 = bi;
    if (pB0 == INT_MAX) return kAtomCapacity;
    const float4 B = sh.pl[pB0];
    const float4 v = make_float4(A.y * B.z - A.z * B.y, A.z * B.x - A.x * B.z, A.x * B.y - A.y * B.x, 0.0f);
    float ptA[3];
    solve3(A, B, v, ptA);
    bv = 9.9e9f;
    bi = INT_MAX;
    for (int c = lane; c < NC + 4; c += 32) {
        if (c == pA0 || c == pB0) continue;
        const float4 C = sh.pl[c];
        const float den = C.x * v.x + C.y * v.y + C.z * v.z;
        if (den != 0.0f) {
            const float vt = fabsf(-(C.x * ptA[0] + C.y * ptA[1] + C.z * ptA[2] + C.w) / den);
            if (vt < bv) { bv = vt; bi = c; }
        }
    }
    warp_argmin(bv, bi);
    const int pC0 = bi;
    if (pC0 == INT_MAX) return kAtomCapacity;
    if (lane == 0) {
        float t[3];
        solve3(sh.pl[pA0], sh.pl[pB0], sh.pl[pC0], t);
        sh.vx[0] = make_float4(t[0], t[1], t[2], sqrtf(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]));
        sh.vp[0] = make_uchar4((uint8_t)pA0, (uint8_t)pB0, (uint8_t)pC0, 0);
        sh.flag[pA0] |= kOnHull;
        sh.flag[pB0] |= kOnHull;
        sh.flag[pC0] |= kOnHull;
        add_edge(sh, 0, pA0, pB0, pC0, 0);
        add_edge(sh, 1, pB0, pC0, pA0, 0);
        add_edge(sh, 2, pC0, pA0, pB0, 0);
    }
    __syncwarp();

    // ---- hull walk (LIB/Vcontacts.cpp:262-410) ----
    int edgenum = 3, startedge = 0, vn = 1;
    for (;;) {
        while (startedge < edgenum && sh.u.e.es[startedge].y != kNone) ++startedge;
        if (startedge >= edgenum) break;
        const uchar4 ep = sh.u.e.ep[startedge];
        const float4 V = sh.u.e.ev[startedge];
        const float4 s = sh.vx[sh.u.e.es[startedge].x];
        const int pA = ep.x, pB = ep.y, oldC = ep.z;
        float vtmin = 9.9e9f;
        int pC = INT_MAX;
        for (int c = lane; c < NC; c += 32) {
            if (c == pA || c == pB || c == oldC) continue;
            const float4 P = sh.pl[c];
            const float den = P.x * V.x + P.y * V.y + P.z * V.z;
            if (den != 0.0f) {
                const float vt = -(P.x * s.x + P.y * s.y + P.z * s.z + P.w) / den;
                if (vt < vtmin && vt > 0.0f) { vtmin = vt; pC = c; }
            }
        }
        warp_argmin(vtmin, pC);
        float x = s.x + vtmin * V.x, y = s.y + vtmin * V.y, z = s.z + vtmin * V.z;
        if (x * x + y * y + z * z > rr) {
            float bvt = vtmin;
            int bc = pC;
            if (lane < 4) {
                const int c = NC + lane;
                if (c != pA && c != pB && c != oldC) {
                    const float4 P = sh.pl[c];
                    const float den = P.x * V.x + P.y * V.y + P.z * V.z;
                    if (den != 0.0f) {
                        const float vt = -(P.x * s.x + P.y * s.y + P.z * s.z + P.w) / den;
                        if (vt < bvt && vt > 0.0f) { bvt = vt; bc = c; }
                    }
                }
            }
            warp_argmin(bvt, bc);
            vtmin = bvt;
            pC = bc;
            x = s.x + vtmin * V.x;
            y = s.y + vtmin * V.y;
            z = s.z + vtmin * V.z;
        }
        if (pC == INT_MAX) return kAtomHullFail;
        if (vn >= kMaxVerts - 1) return kAtomCapacity;
        // edges (pA, pC) and (pB, pC): the first open match after startedge, else a new edge
        int mAC = INT_MAX, mBC = INT_MAX;
        for (int e0 = startedge + 1; e0 < edgenum; e0 += 32) {
            const int e = e0 + lane;
            bool ac = false, bc = false;
            if (e < edgenum) {
                const uchar4 q = sh.u.e.ep[e];
                ac = (q.x == pA && q.y == pC) || (q.x == pC && q.y == pA);
                bc = (q.x == pB && q.y == pC) || (q.x == pC && q.y == pB);
            }
            const unsigned ma = __ballot_sync(kFull, ac), mb = __ballot_sync(kFull, bc);
            if (ma && mAC == INT_MAX) mAC = e0 + __ffs(ma) - 1;
            if (mb && mBC == INT_MAX) mBC = e0 + __ffs(mb) - 1;
        }
        if (lane == 0) {
            sh.vx[vn] = make_float4(x, y, z, sqrtf(x * x + y * y + z * z));
            sh.vp[vn] = make_uchar4((uint8_t)pA, (uint8_t)pB, (uint8_t)pC, 0);
            sh.u.e.es[startedge].y = (uint8_t)vn;
            sh.u.e.ep[startedge].w = (uint8_t)pC;
            sh.flag[pC] |= kOnHull;
        }
        __syncwarp();
        if (mAC != INT_MAX) {
            if (lane == 0) {
                sh.u.e.es[mAC].y = (uint8_t)vn;
                sh.u.e.ep[mAC].w = (uint8_t)pB;
            }
        } else {
            if (lane == 0) add_edge(sh, edgenum, pA, pC, pB, vn);
            ++edgenum;
        }
        __syncwarp();
        if (mBC != INT_MAX) {
            if (lane == 0) {
                sh.u.e.es[mBC].y = (uint8_t)vn;
                sh.u.e.ep[mBC].w = (uint8_t)pA;
            }
        } else {
            if (lane == 0) add_edge(sh, edgenum, pB, pC, pA, vn);
            ++edgenum;
            if (edgenum >= kMaxEdges) return kAtomHullFail;
        }
        __syncwarp();
        ++vn;
    }

    // ---- arc points where edges leave the sphere (LIB/Vcontacts.cpp:418-462) ----
    for (int e0 = 0; e0 < edgenum; e0 += 32) {
        const int e = e0 + lane;
        int cnt = 0;
        float a0[3], a1[3];
        bool k0 = false, k1 = false;
        uchar4 q = make_uchar4(0, 0, 0, 0);
        if (e < edgenum) {
            q = sh.u.e.ep[e];
            const uchar2 se = sh.u.e.es[e];
            if (rado < sh.vx[se.x].w || rado < sh.vx[se.y].w) {
                if (solve2s(sh.pl[q.x], sh.pl[q.y], rado, a0, a1)) {
                    const float4 ta = sh.pl[q.z], tb = sh.pl[q.w];
                    k0 = (dot3(ta, a0[0], a0[1], a0[2]) + ta.w < 0.0f) && (dot3(tb, a0[0], a0[1], a0[2]) + tb.w < 0.0f);
                    k1 = (dot3(ta, a1[0], a1[1], a1[2]) + ta.w < 0.0f) && (dot3(tb, a1[0], a1[1], a1[2]) + tb.w < 0.0f);
                    cnt = (int)k0 + (int)k1;
                }
            }
        }
        int tot;
        const int off = warp_excl_scan(cnt, lane, &tot);
        if (vn + tot > kMaxVerts - 1) return kAtomCapacity;
        int w = vn + off;
        if (k0) {
            sh.vx[w] = make_float4(a0[0], a0[1], a0[2], rado);
            sh.vp[w] = make_uchar4(q.x, q.y, kNone, 0);
            ++w;
        }
        if (k1) {
            sh.vx[w] = make_float4(a1[0], a1[1], a1[2], rado);
            sh.vp[w] = make_uchar4(q.x, q.y, kNone, 0);
        }
        vn += tot;
        __syncwarp();
    }
    // ---- keep the vertices inside the sphere, in order ----
    int nv = 0;
    for (int v0 = 0; v0 < vn; v0 += 32) {
        const int vi = v0 + lane;
        float4 X = make_float4(0, 0, 0, 0);
        uchar4 P = make_uchar4(0, 0, 0, 0);
        bool keep = false;
        if (vi < vn) {
            X = sh.vx[vi];
            P = sh.vp[vi];
            keep = X.w <= rado;
        }
        const unsigned m = __ballot_sync(kFull, keep);
        __syncwarp();
        if (keep) {
            const int w = nv + __popc(m & lanemask_lt());
            sh.vx[w] = X;
            sh.vp[w] = P;
        }
        nv += __popc(m);
        __syncwarp();
    }
    const int NV = nv;

    // ---- faces: points per plane in vertex order, plus an antipodal arc point ----
    // (the edge arrays are dead from here on; their storage holds the face lists)
    int tot_pts = 0;
    for (int x0 = 0; x0 < NC; x0 += 32) {
        const int X = x0 + lane;
        int cnt = 0;
        if (X < NC && sh.flag[X] != 0)
            for (int vi = 0; vi < NV; ++vi) {
                const uchar4 P = sh.vp[vi];
                cnt += (P.x == X || P.y == X || P.z == X);
            }
        const int need = cnt + (cnt > 2 ? 1 : 0);
        int t;
        const int off = warp_excl_scan(need, lane, &t);
        if (X < NC) {
            sh.foff[X] = (uint16_t)(tot_pts + off);
            sh.fnp[X] = (uint8_t)min(cnt, 255);
        }
        tot_pts += t;
    }
    if (tot_pts > kMaxFacePts) return kAtomCapacity;
    __syncwarp();
    int n_extra = 0;
    for (int x0 = 0; x0 < NC; x0 += 32) {
        const int X = x0 + lane;
        bool extra = false;
        float ex[3] = {0.f, 0.f, 0.f};
        if (X < NC && sh.flag[X] != 0) {
            const int o = sh.foff[X];
            int k = 0;
            for (int vi = 0; vi < NV; ++vi) {
                const uchar4 P = sh.vp[vi];
                if (P.x == X || P.y == X || P.z == X) sh.u.f.pt[o + k++] = (uint8_t)vi;
            }
            if (k > 2) {
                const float4 cp = centre_of(sh.pl[X]);
                for (int q = 0; q < k; ++q) {
                    const int vi = sh.u.f.pt[o + q];
                    if (sh.vp[vi].z == kNone) {
                        const float4 pv = sh.vx[vi];
                        ex[0] = 2.0f * cp.x - pv.x;
                        ex[1] = 2.0f * cp.y - pv.y;
                        ex[2] = 2.0f * cp.z - pv.z;
                        extra = inside_all(sh, NC, X, ex[0], ex[1], ex[2]);
                        break;
                    }
                }
            }
        }
        int t;
        const int off = warp_excl_scan(extra ? 1 : 0, lane, &t);
        if (NV + n_extra + t > kMaxVerts - 1) return kAtomCapacity;
        if (extra) {
            const int w = NV + n_extra + off;
            sh.vx[w] = make_float4(ex[0], ex[1], ex[2], rado);
            sh.vp[w] = make_uchar4((uint8_t)X, kNone, kNone, 0);
            sh.u.f.pt[sh.foff[X] + sh.fnp[X]] = (uint8_t)w;
            sh.fnp[X] += 1;
        }
        n_extra += t;
    }
    __syncwarp();
    // ordering around each face (pt[0], a neighbour of it, then decreasing cosine)
    int np_miss = 0;
    for (int X = lane; X < NC; X += 32) {
        if (sh.flag[X] == 0) continue;
        const int np = sh.fnp[X];
        if (np <= 3) continue;
        uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
        float* cs = &sh.u.f.cosv[sh.foff[X]];
        const uchar4 P0 = sh.vp[pt[0]];
        const int pY = (P0.x == X) ? P0.y : P0.x;
        int vi = 1;
        for (; vi < np; ++vi) {
            const uchar4 q = sh.vp[pt[vi]];
            if (q.x == pY || q.y == pY || q.z == pY) break;
        }
        if (vi == np) {
            ++np_miss;
            const int pZ = (P0.x == X || P0.y == X) ? P0.z : P0.y;
            vi = 1;
            if (pZ != kNone) {
                int w = 1;
                for (; w < np; ++w) {
                    const uchar4 q = sh.vp[pt[w]];
                    if (q.x == pZ || q.y == pZ || q.z == pZ) break;
                }
                if (w < np) vi = w;
            }
        }
        const uint8_t tmp = pt[vi];
        pt[vi] = pt[1];
        pt[1] = tmp;
        const float4 v0 = sh.vx[pt[0]], v1 = sh.vx[pt[1]];
        for (int k = 2; k < np; ++k) cs[k] = cos_pqr(v1, v0, sh.vx[pt[k]]);
        for (int a = 2; a < np - 1; ++a)
            for (int b = a + 1; b < np; ++b)
                if (cs[a] < cs[b]) {
                    const uint8_t t = pt[a];
                    pt[a] = pt[b];
                    pt[b] = t;
                    const float tc = cs[a];
                    cs[a] = cs[b];
                    cs[b] = tc;
                }
    }
    *no_partner += warp_sum(np_miss);
    __syncwarp();

    // ---- areas (LIB/Vcontacts.cpp:838-1044) ----
    // the first three engulfing planes in plane order
    int epi = 0;
    for (int x0 = 0; x0 < NC && epi < 3; x0 += 32) {
        const int X = x0 + lane;
        const unsigned m = __ballot_sync(kFull, X < NC && (sh.flag[X] & kEngulf));
        unsigned mm = m;
        while (mm && epi < 3) {
            const int b = __ffs(mm) - 1;
            mm &= mm - 1;
            if (lane == 0) sh.eng[epi] = x0 + b;
            ++epi;
        }
    }
    __syncwarp();
    if (epi > 0) {
        // project_points (LIB/Vcontacts.cpp:1278-1344)
        float pp[3];
        if (epi == 1) {
            const float4 c = centre_of(sh.pl[sh.eng[0]]);
            pp[0] = c.x; pp[1] = c.y; pp[2] = c.z;
        } else if (epi == 2) {
            float q0[3], q1[3];
            if (!solve2s(sh.pl[sh.eng[0]], sh.pl[sh.eng[1]], rado, q0, q1)) {
                pp[0] = sh.vx[kMaxVerts - 1].x;   // atom-centre fallback, staged by the caller
                pp[1] = sh.vx[kMaxVerts - 1].y;
                pp[2] = sh.vx[kMaxVerts - 1].z;
            } else {
                pp[0] = (q0[0] + q1[0]) / 2; pp[1] = (q0[1] + q1[1]) / 2; pp[2] = (q0[2] + q1[2]) / 2;
            }
        } else {
            solve3(sh.pl[sh.eng[0]], sh.pl[sh.eng[1]], sh.pl[sh.eng[2]], pp);
        }
        for (int vi = lane; vi < NV; vi += 32) {
            if (sh.vp[vi].z == kNone) continue;
            float4 P = sh.vx[vi];
            const float Vx = P.x - pp[0], Vy = P.y - pp[1], Vz = P.z - pp[2];
            const float a = Vx * Vx + Vy * Vy + Vz * Vz;
            const float b = 2 * (P.x * Vx + P.y * Vy + P.z * Vz);
            const float c = P.x * P.x + P.y * P.y + P.z * P.z - rado * rado;
            const float k = (sqrtf(b * b - 4.0f * a * c) - b) / (2 * a);
            P.x += k * Vx; P.y += k * Vy; P.z += k * Vz;
            P.w = rado;
            sh.vx[vi] = P;
        }
        __syncwarp();
    }
    const float two_pi_r = 2.0f * (float)kPi * rado;
    for (int X = lane; X < NC; X += 32) {
        if (sh.flag[X] == 0) continue;
        const int np = sh.fnp[X];
        const uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
        const float4 cp = centre_of(sh.pl[X]);
        float area = 0.0f;
        if (np == 0) {
            if (inside_all(sh, NC, X, cp.x, cp.y, cp.z)) area = two_pi_r * (rado - cp.w);
        } else if (np == 2) {
            const float arc = sph_arc(cp, sh.vx[pt[0]], sh.vx[pt[1]], rado);
            if (inside_all(sh, NC, X, cp.x, cp.y, cp.z)) area = two_pi_r * (rado - cp.w) - arc;
            else area = arc;
        } else {
            const float4 v0 = sh.vx[pt[0]];
            float cN0_prev = 0.0f;
            for (int vi = 1; vi < np - 1; ++vi) {
                const float4 va = sh.vx[pt[vi]], vb = sh.vx[pt[vi + 1]];
                const float cNN1 = (va.x * vb.x + va.y * vb.y + va.z * vb.z) / (va.w * vb.w);
                const float cN0a = vi == 1 ? (v0.x * va.x + v0.y * va.y + v0.z * va.z) / (v0.w * va.w) : cN0_prev;
                const float cN0b = (v0.x * vb.x + v0.y * vb.y + v0.z * vb.z) / (v0.w * vb.w);
                cN0_prev = cN0b;
                const float U = sqrtf((1 + cN0a) * (1 + cNN1) * (1 + cN0b) / 8.0f);
                const float V = sqrtf((1 - cN0a) * (1 - cNN1) * (1 + cN0b) / 8.0f);
                const float W = sqrtf((1 - cN0a) * (1 + cNN1) * (1 - cN0b) / 8.0f);
                const float Xv = sqrtf((1 + cN0a) * (1 - cNN1) * (1 - cN0b) / 8.0f);
                const float tS = (1 - U + V + W + Xv) / (1 + U - V - W - Xv);
                const float tSA = (1 - U - V - W + Xv) / (1 + U + V + W - Xv);
                const float tSB = (1 - U - V + W - Xv) / (1 + U + V - W + Xv);
                const float tSC = (1 - U + V - W - Xv) / (1 + U - V + W + Xv);
                const float tanprod = sqrtf(tS * tSA * tSB * tSC);
                if (tanprod > 0.0f) area += 4.0f * rado * rado * atanf(sqrtf(tanprod));
            }
            for (int vi = 0; vi < np; ++vi) {
                const int a = pt[vi], b = pt[(vi + 1) % np];
                const uchar4 qa = sh.vp[a], qb = sh.vp[b];
                if (qa.z == kNone && qb.z == kNone) {
                    const int sa = (qa.y == kNone ? -1 : qa.y) + qa.x;
                    const int sb = (qb.y == kNone ? -1 : qb.y) + qb.x;
                    if (sa != sb) area += sph_arc(cp, sh.vx[a], sh.vx[b], rado);
                }
            }
        }
        sh.area[X] = area;
    }
    __syncwarp();
    if (epi > 0) {
        if (lane == 0) {
            for (int X = 0; X < NC; ++X) {
                if (!(sh.flag[X] & kEngulf)) continue;
                const int np = sh.fnp[X];
                const uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
                const float4 cp = centre_of(sh.pl[X]);
                for (int vi = 0; vi < np; ++vi) {
                    const int cur = pt[vi], nxt = pt[(vi + 1) % np];
                    const uchar4 qc = sh.vp[cur], qn = sh.vp[nxt];
                    int pa1, pa2;
                    if (qc.x == X) { pa1 = qc.y; pa2 = qc.z; }
                    else { pa1 = qc.x; pa2 = (qc.y == X) ? qc.z : qc.y; }
                    int comm;
                    if (pa1 == qn.x || pa1 == qn.y || pa1 == qn.z) comm = pa1;
                    else if (pa2 == qn.x || pa2 == qn.y || pa2 == qn.z) comm = pa2;
                    else continue;
                    if (comm != kNone && !(comm < NC && (sh.flag[comm] & kEngulf))) {
                        if (comm < NC) sh.area[comm] += sph_arc(cp, sh.vx[cur], sh.vx[nxt], rado);
                        if (np == 2) break;
                    }
                }
            }
            if (epi == 1) {
                sh.area[sh.eng[0]] = two_pi_r * (rado + fabsf(sh.pl[sh.eng[0]].w));
            } else if (epi == 2) {
                float q0[3], q1[3];
                const float full = two_pi_r * rado;
                if (!solve2s(sh.pl[sh.eng[0]], sh.pl[sh.eng[1]], rado, q0, q1)) {
                    sh.area[sh.eng[0]] = full;
                    sh.area[sh.eng[1]] = full;
                } else {
                    const float4 Bp = make_float4(q0[0], q0[1], q0[2], rado);
                    const float4 Cp = make_float4(q1[0], q1[1], q1[2], rado);
                    float m = sph_arc(centre_of(sh.pl[sh.eng[0]]), Bp, Cp, rado);
                    m += sph_arc(centre_of(sh.pl[sh.eng[1]]), Bp, Cp, rado);
                    sh.area[sh.eng[0]] = full - 0.5f * m;
                    sh.area[sh.eng[1]] = full - 0.5f * m;
                }
            }
        }
        __syncwarp();
        if (epi >= 3) {
            const float share = 4.0f * (float)kPi * rado * rado / epi;
            for (int X = lane; X < NC; X += 32) sh.area[X] = (sh.flag[X] & kEngulf) ? share : 0.0f;
        }
        __syncwarp();
    }
    // a face reaches the sphere when it has points there or a non-zero area
    for (int X = lane; X < NC; X += 32)
        if (sh.flag[X] != 0 && (sh.fnp[X] > 0 || sh.area[X] != 0.0f)) sh.flag[X] |= kTouches;
    sh.nv = NV;
    __syncwarp();
    return kAtomOk;
}

// Planes of the candidates of one ligand atom (LIB/Vcontacts.cpp:186-221). Slots set in
// `excl` (a candidate the reference would not see) get a plane that never binds.
__device__ void load_planes(VorShared& sh, const DevSystem& S, const DevWork& W, int p, int a,
                            int NC, float4 me, float rado, const uint32_t* excl, int lane) {
    const size_t cb = ((size_t)p * S.n_lig + a) * kMaxCand;
    const float rr = rado * rado;
    for (int c = lane; c < NC; c += 32) {
        const int j = W.cand_idx[cb + c];
        const float d2 = W.cand_d2[cb + c];
        sh.cidx[c] = j;
        const float4 pj = j < S.n_rec ? S.rec_pos[j] : W.lig_pos[(size_t)p * S.n_lig + (j - S.n_rec)];
        const bool ex = (excl && ((excl[c >> 5] >> (c & 31)) & 1u)) || d2 < 1e-20f;
        if (ex) {
            sh.pl[c] = make_float4(0.0f, 0.0f, 0.0f, -1e30f);
            sh.flag[c] = 0;
            continue;
        }
        const float d = sqrtf(d2);
        const float q = kRw + pj.w;
        const float num = (d2 + rr) - q * q;
        bool eng = num < 0.0f;
        if (fabsf(num) < 1e-3f) eng = ((double)d2 + (double)rr) - (double)(q * q) < 0.0;
        sh.pl[c] = make_float4((pj.x - me.x) / d, (pj.y - me.y) / d, (pj.z - me.z) / d, -(num / (2.0f * d)));
        sh.flag[c] = eng ? kEngulf : 0;
    }
    if (lane == 0) sh.vx[kMaxVerts - 1] = make_float4(me.x + rado, me.y, me.z, 0.0f);
    __syncwarp();
}

__device__ void store_results(VorShared& sh, const DevSystem& S, const DevWork& W, int p, int a,
                              int NC, int status, int lane) {
    const size_t cb = ((size_t)p * S.n_lig + a) * kMaxCand;
    uint32_t mask[kMaskWords] = {0, 0, 0, 0};
    for (int c = lane; c < NC; c += 32) {
        const float ar = status == kAtomOk ? sh.area[c] : 0.0f;
        const uint8_t f = status == kAtomOk ? sh.flag[c] : 0;
        W.cand_area[cb + c] = ar;
        W.cand_flag[cb + c] = f;
        const int j = sh.cidx[c];
        if (j >= S.n_rec && ar > 0.0f && (f & (kOnHull | kEngulf))) {
            const int l = j - S.n_rec;
            mask[l >> 5] |= 1u << (l & 31);
        }
    }
#pragma unroll
    for (int w = 0; w < kMaskWords; ++w) {
        uint32_t m = mask[w];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m |= __shfl_xor_sync(kFull, m, o);
        if (lane == 0 && w * 32 < S.n_lig) W.rec0[((size_t)p * S.n_lig + a) * kMaskWords + w] = m;
    }
    if (lane == 0) W.atom_status[(size_t)p * S.n_lig + a] = status;
}

__device__ double pose_clash_sum(const DevSystem& S, const DevWork& W, int p, int lane) {
    double s = 0.0;
    for (int l = lane; l < S.n_lig; l += 32) s += W.clash_part[(size_t)p * S.n_lig + l];
    return warp_sum(s);
}

// ------------------------------------------------------------------------------------------
// contacts_kernel
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
contacts_kernel(DevSystem S, DevWork W, int n) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int nl = S.n_lig;
    if (gw >= n * nl) return;
    const int p = gw / nl, a = gw % nl;
    const size_t lb = (size_t)p * nl;
    const int4 pg = W.pose_grid[p];
    const size_t cb = (lb + a) * kMaxCand;
    if (pg.z) {  // the pose left the grid the reference can index
        if (lane == 0) {
            W.cand_n[lb + a] = 0;
            W.clash_part[lb + a] = 0.0;
        }
        return;
    }
    const float4 me = W.lig_pos[lb + a];
    const float rado = me.w + kRw;
    const int my_rank = W.lig_rank[lb + a];
    const int dim = pg.y, dim2 = dim * dim, dim3 = dim2 * dim;
    const int box0 = W.lig_cell[lb + a];
    // ligand atoms held by this lane (atom lane + 32 * slot): cell offset key 0..26 or -1
    int key[kMaxLig / 32];
    float4 lpos[kMaxLig / 32];
#pragma unroll
    for (int s = 0; s < kMaxLig / 32; ++s) {
        const int l = lane + 32 * s;
        key[s] = -1;
        lpos[s] = make_float4(0, 0, 0, 0);
        if (l < nl) {
            lpos[s] = W.lig_pos[lb + l];
            const int o = W.lig_cell[lb + l] - box0 + dim2 + dim + 1;
            if (o >= 0) {
                const int di = o / dim2, rem = o - di * dim2, dj = rem / dim, dk = rem - dj * dim;
                if (di <= 2 && dj <= 2 && dk <= 2) key[s] = di * 9 + dj * 3 + dk;
            }
        }
    }
    const float4 gm = W.pose_gmin[p];
    int nc = 0;
    double clash = 0.0;
    const double permea = (double)S.permeability;
    bool overflow = false;
    auto consider = [&](bool in, int j, float4 pj) {
        bool pass = false;
        float sq = 0.0f;
        if (in) {
            const float dx = __fsub_rn(me.x, pj.x), dy = __fsub_rn(me.y, pj.y), dz = __fsub_rn(me.z, pj.z);
            sq = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            const float nd = __fadd_rn(__fadd_rn(rado, pj.w), kRw);
            pass = ((double)sq < (double)nd * (double)nd) && sq != 0.0f;
        }
        const unsigned m = __ballot_sync(kFull, pass);
        if (pass) {
            const int w = nc + __popc(m & lanemask_lt());
            if (w < kMaxCand) {
                W.cand_idx[cb + w] = j;
                W.cand_d2[cb + w] = sq;
            }
            // clash pre-filter share: receptor partners, and ligand partners processed later
            const bool later = j < S.n_rec || W.lig_rank[lb + (j - S.n_rec)] > my_rank;
            if (later) {
                const double rAB = (double)__fadd_rn(me.w, pj.w);
                const double cd = permea * rAB;
                const double dist = sqrt((double)sq);
                if (dist < cd) {
                    const bool intra = j >= S.n_rec;
                    if (!intra || S.bonded[a * nl + (j - S.n_rec)] < 0)
                        clash += (double)kKwall * (pow(dist, -12.0) - pow(cd, -12.0));
                }
            }
        }
        nc += __popc(m);
    };
    for (int i = 0; i < 27; ++i) {
        const int bi = box0 + dim2 * ((i / 9) - 1) + dim * (((i / 3) % 3) - 1) + (i % 3) - 1;
        if (bi < 0 || bi >= dim3) continue;
        if (!pg.x) {
            const int s0 = S.cell_start[bi], s1 = S.cell_start[bi + 1];
            for (int k0 = s0; k0 < s1; k0 += 32) {
                const int k = k0 + lane;
                const bool in = k < s1;
                const int j = in ? S.cell_atom[k] : 0;
                const float4 pj = in ? S.cell_pos[k] : make_float4(0, 0, 0, 0);
                consider(in, j, pj);
            }
        } else {
            // a grid re-derived for this pose: scan every receptor atom for cell bi
            for (int k0 = 0; k0 < S.n_rec; k0 += 32) {
                const int k = k0 + lane;
                bool in = false;
                float4 pj = make_float4(0, 0, 0, 0);
                if (k < S.n_rec) {
                    pj = S.rec_pos[k];
                    const int cb2 = (int)((pj.x - gm.x) / kCell) * dim2 + (int)((pj.y - gm.y) / kCell) * dim +
                                    (int)((pj.z - gm.z) / kCell);
                    in = cb2 == bi;
                }
                consider(in, k, pj);
            }
        }
#pragma unroll
        for (int s = 0; s < kMaxLig / 32; ++s) {
            if (32 * s >= nl) break;
            consider(key[s] == i, S.n_rec + lane + 32 * s, lpos[s]);
        }
    }
    overflow = nc > kMaxCand;
    clash = warp_sum(clash);
    if (lane == 0) {
        W.cand_n[lb + a] = overflow ? -nc : nc;
        W.clash_part[lb + a] = clash;
    }
}

// ------------------------------------------------------------------------------------------
// voronoi_kernel
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kVorWarps * 32)
voronoi_kernel(DevSystem S, DevWork W, int n) {
    extern __shared__ __align__(16) unsigned char smem[];
    VorShared& sh = reinterpret_cast<VorShared*>(smem)[threadIdx.x >> 5];
    const int gw = blockIdx.x * kVorWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const int nl = S.n_lig;
    if (gw >= n * nl) return;
    const int p = gw / nl, a = gw % nl;
    const size_t lb = (size_t)p * nl;
    const int NC = W.cand_n[lb + a];
    int status;
    if (W.pose_grid[p].z || pose_clash_sum(S, W, p, lane) >= kClashThreshold) {
        status = kAtomSkipped;
    } else if (NC < 0) {
        status = kAtomCapacity;
    } else if (NC == 0) {
        status = kAtomOk;
    } else {
        const float4 me = W.lig_pos[lb + a];
        const float rado = me.w + kRw;
        load_planes(sh, S, W, p, a, NC, me, rado, nullptr, lane);
        int np_miss = 0;
        status = voronoi_warp(sh, NC, rado, lane, &np_miss);
        if (lane == 0 && np_miss) atomicAdd(&W.counters[3], np_miss);
    }
    store_results(sh, S, W, p, a, status == kAtomSkipped || NC < 0 ? 0 : NC, status, lane);
}

// ------------------------------------------------------------------------------------------
// score_kernel
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ bool bit(const uint32_t* m, int l) { return (m[l >> 5] >> (l & 31)) & 1u; }

__device__ double get_yval(const DevSystem& S, int idx, double rel) {
    const int o = S.em_off[idx], e = S.em_off[idx + 1];
    if (S.em_weight[idx]) return (double)S.em_y[o];
    int k = o;
    while (k + 1 < e && rel > (double)S.em_x[k + 1]) ++k;
    if ((double)S.em_x[k] > rel) return 0.0;
    if (k + 1 >= e) return (double)S.em_y[k];
    return (double)S.em_y[k] + (rel - (double)S.em_x[k]) / (double)(S.em_x[k + 1] - S.em_x[k]) *
                                   (double)(S.em_y[k + 1] - S.em_y[k]);
}

__global__ void __launch_bounds__(kVorWarps * 32)
score_kernel(DevSystem S, DevWork W, int n) {
    extern __shared__ __align__(16) unsigned char smem[];
    VorShared& sh = reinterpret_cast<VorShared*>(smem)[threadIdx.x >> 5];
    const int p = blockIdx.x * kVorWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= n) return;
    const int nl = S.n_lig;
    const size_t lb = (size_t)p * nl;
    fxe_cf cf;
    memset(&cf, 0, sizeof(cf));
    if (W.pose_grid[p].z) {
        cf.status = FXE_POSE_CAPACITY;
        if (lane == 0) W.out[p] = cf;
        return;
    }
    const double clash = pose_clash_sum(S, W, p, lane);
    if (clash >= kClashThreshold) {
        cf.wal = clash;
        cf.metal_coord = 1.0;
        cf.evalue = cf.wal + cf.metal_coord;
        cf.status = FXE_POSE_CLASHED;
        if (lane == 0) W.out[p] = cf;
        return;
    }
    // Replay calc_region in Calclist order: atom a keeps a ligand partner j processed before it
    // only if j kept a; when such a dropped partner's plane reaches a's sphere, a is
    // recomputed without the dropped planes, as the reference computes it.
    uint32_t excl[kMaxCand / 32];
    int capacity = 0, fail = 0;
    for (int r = 0; r < nl; ++r) {
        int a = -1;
        for (int l = lane; l < nl; l += 32)
            if (W.lig_rank[lb + l] == r) a = l;
        for (int o = 16; o > 0; o >>= 1) a = max(a, __shfl_xor_sync(kFull, a, o));
        const int st = W.atom_status[lb + a];
        const int NC = W.cand_n[lb + a];
        if (NC < 0 || st == kAtomCapacity) { capacity = 1; break; }
        const size_t cb = (lb + a) * kMaxCand;
        bool need = false;
        bool any_excl = false;
        for (int w = 0; w < kMaxCand / 32; ++w) excl[w] = 0;
        for (int c0 = 0; c0 < NC; c0 += 32) {
            const int c = c0 + lane;
            bool ex = false, touch = false;
            if (c < NC) {
                const int j = W.cand_idx[cb + c];
                if (j >= S.n_rec) {
                    const int l = j - S.n_rec;
                    if (W.lig_rank[lb + l] < r && !bit(&W.rec0[(lb + l) * kMaskWords], a)) {
                        ex = true;
                        touch = (W.cand_flag[cb + c] & (kTouches | kEngulf)) != 0;
                    }
                }
            }
            excl[c0 >> 5] = __ballot_sync(kFull, ex);
            any_excl |= excl[c0 >> 5] != 0;
            need |= __any_sync(kFull, touch);
        }
        if (st == kAtomHullFail && !any_excl) { fail = 1; break; }
        if (need || (st == kAtomHullFail && any_excl)) {
            const float4 me = W.lig_pos[lb + a];
            const float rado = me.w + kRw;
            load_planes(sh, S, W, p, a, NC, me, rado, excl, lane);
            int np_miss = 0;
            const int st2 = voronoi_warp(sh, NC, rado, lane, &np_miss);
            store_results(sh, S, W, p, a, NC, st2, lane);
            if (lane == 0) atomicAdd(&W.counters[0], 1);
            if (st2 == kAtomCapacity) { capacity = 1; break; }
            if (st2 == kAtomHullFail) { fail = 1; break; }
            __syncwarp();
        }
    }
    if (capacity || fail) {
        if (capacity) {
            cf.status = FXE_POSE_CAPACITY;
            if (lane == 0) atomicAdd(&W.counters[2], 1);
        } else {
            cf.wal = (double)kPolyPenalty;
            cf.metal_coord = 1.0;
            cf.evalue = cf.wal + cf.metal_coord;
            cf.status = FXE_POSE_POLYHEDRON_FAILED;
            if (lane == 0) atomicAdd(&W.counters[1], 1);
        }
        if (lane == 0) W.out[p] = cf;
        return;
    }
    // vcfunction: atoms in Calc order, their kept contacts
    const int T = S.ntypes;
    const double permea = (double)S.permeability;
    double com = 0.0, wal = 0.0, sas = 0.0, totsas = 0.0;
    for (int i = 0; i < nl; ++i) {
        const int NC = W.cand_n[lb + i];
        const size_t cb = (lb + i) * kMaxCand;
        const int ri = W.lig_rank[lb + i];
        const double radA = (double)S.lig_radius[i];
        const double radoA = radA + (double)kRw;
        const double surfA = 4.0 * kPi * radoA * radoA;
        const int ti = S.lig_type[i];
        double c_com = 0.0, c_wal = 0.0, c_area = 0.0;
        for (int c = lane; c < NC; c += 32) {
            const int j = W.cand_idx[cb + c];
            const float ar = W.cand_area[cb + c];
            uint8_t f = W.cand_flag[cb + c];
            bool kept = ar > 0.0f && (f & (kOnHull | kEngulf));
            const bool lig = j >= S.n_rec;
            const int l = j - S.n_rec;
            if (kept && lig && W.lig_rank[lb + l] < ri) kept = bit(&W.rec0[(lb + l) * kMaskWords], i);
            if (kept) W.cand_flag[cb + c] = f | kRecorded;
            if (!kept) continue;
            const double area = (double)ar;
            c_area += area;
            if (lig && (S.bonded[l * nl + i] >= 0 || l < i)) continue;
            const float rj = lig ? S.lig_radius[l] : S.rec_pos[j].w;
            const int tj = lig ? S.lig_type[l] : S.rec_type[j];
            const int eidx = (ti - 1) * T + (tj - 1);
            const double yval = get_yval(S, eidx, area / surfA);
            c_com += S.em_weight[eidx] ? yval * area : yval;
            const double rAB = radA + (double)rj;
            const float clash_distance = (float)(permea * rAB);
            const float d2 = W.cand_d2[cb + c];
            if (d2 < clash_distance * clash_distance * 1.0001f) {
                const double dd = sqrt((double)d2);
                if (dd < (double)clash_distance) {
                    const double q2 = dd * dd, q4 = q2 * q2, q6 = q4 * q2;
                    const double cr = permea * rAB;
                    const double r2 = cr * cr, r4 = r2 * r2, r6 = r4 * r2;
                    c_wal += (double)kKwall * (1.0 / (q6 * q6) - 1.0 / (r6 * r6));
                }
            }
        }
        c_com = warp_sum(c_com);
        c_wal = warp_sum(c_wal);
        c_area = warp_sum(c_area);
        double SAS = surfA - c_area;
        if (SAS < 0.0) SAS = 0.0;
        totsas += SAS;
        double contribution;
        if (S.solventterm != 0.0f) {
            contribution = (double)S.solventterm * SAS;
        } else {
            const int eidx = (ti - 1) * T + (T - 1);
            const double yval = get_yval(S, eidx, SAS / surfA);
            contribution = S.em_weight[eidx] ? yval * SAS : yval;
        }
        com += c_com;
        wal += c_wal;
        sas += contribution;
    }
    cf.com = com;
    cf.wal = wal;
    cf.sas = sas;
    cf.totsas = totsas;
    cf.evalue = cf.com + cf.wal + cf.sas + cf.con + cf.elec + cf.hbond + cf.gist_desolv + cf.metal_coord;
    cf.status = FXE_POSE_SCORED;
    if (lane == 0) W.out[p] = cf;
}

size_t voronoi_smem_bytes() { return sizeof(VorShared) * kVorWarps; }

void launch_contacts(const DevSystem& S, const DevWork& W, int n, cudaStream_t st) {
    const long warps = (long)n * S.n_lig;
    contacts_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, st>>>(S, W, n);
}

void launch_voronoi(const DevSystem& S, const DevWork& W, int n, cudaStream_t st) {
    const long warps = (long)n * S.n_lig;
    voronoi_kernel<<<(unsigned)((warps + kVorWarps - 1) / kVorWarps), kVorWarps * 32,
                     voronoi_smem_bytes(), st>>>(S, W, n);
}

void launch_score(const DevSystem& S, const DevWork& W, int n, cudaStream_t st) {
    score_kernel<<<(unsigned)((n + kVorWarps - 1) / kVorWarps), kVorWarps * 32,
                   voronoi_smem_bytes(), st>>>(S, W, n);
}

cudaError_t configure_voronoi() {
    cudaError_t e = cudaFuncSetAttribute(voronoi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)voronoi_smem_bytes());
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(score_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)voronoi_smem_bytes());
}

}  // namespace fxe
