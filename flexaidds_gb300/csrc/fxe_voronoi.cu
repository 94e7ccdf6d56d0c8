// fxe_voronoi.cu — Voronoi contact surfaces and complementarity scoring (the candidate lists
// come from contacts_kernel, fxe_contacts.cu).
//
// pose_kernel      one warp per pose: calc_region's loop over the scorable atoms in Calclist
//                  order (LIB/Vcontacts.cpp:74-139) — each atom's list without the saved atoms
//                  that kept no contact with it, its extended-radical-plane polyhedron started
//                  from the seed an earlier atom left (voronoi_poly2, :147-490), faces
//                  (order_faces, :699-831) and spherical areas (calc_areas, :838-1044) in FP64
//                  (reference precision) or FP32 (fast precision), the contacts it keeps
//                  (save_areas) and the seeds it leaves (save_seeds) —
//                  then vcfunction's walk over the kept contacts (LIB/vcfunction.cpp:14-574).
//
// The atoms of one pose stay in order because the reference's results depend on it: which
// earlier atom seeds a hull decides the walk's start vertex, and with engulfing planes the
// atom centre lies outside its own cell, so a start from the closest plane can lie outside the
// cell and trace another polyhedron. Parallelism is across poses (one warp each) and across
// the planes, edges, vertices and faces of each polyhedron (the 32 lanes).
#include <cfloat>
#include <climits>

#include "fxe_common.cuh"

namespace fxe {
namespace FXE_VARIANT {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kFaceWords = (kMaxCand + 31) / 32;
constexpr uint8_t kNone = 255;

// Floating-point type of the polyhedron arithmetic: single precision by default; building
// with -DFXE_REAL=double gives the same algorithm in double precision (for comparisons).
#ifndef FXE_REAL
#define FXE_REAL float
#endif
#ifndef FXE_VARIANT
#define FXE_VARIANT f32
#endif
using real = FXE_REAL;
// Double builds evaluate the areas with the reference's own expressions (they are not well
// conditioned for small or nearly degenerate triangles, and the double build reproduces the
// reference's values there too); single builds use well-conditioned equivalents.
#ifndef FXE_REFERENCE_FORMULAS
#define FXE_REFERENCE_FORMULAS 0
#endif
// Double builds decide the hull walk's plane tests in single precision first and redo a test
// in double only when its single-precision result is within its error bound of deciding the
// other way (see walk_step_group).
#ifndef FXE_FILTER
#define FXE_FILTER (FXE_REFERENCE_FORMULAS)
#endif
// Poses (warps) per block of pose_kernel, and whether the block's warps meet after every atom.
// The double kernel's code (about 220 KB) outgrows the SM's instruction caches, and its top stall
// was instruction fetch with eight warps of an SM at unrelated points of it: eight warps per block
// (one block per SM, 20 KB of workspace each) that take eight neighbouring poses of the queue and
// meet at a block barrier after each atom fetch the same code at about the same time (measured on
// GB300, plain-scale workload: 22.9 -> 19.2 ms per launch; four warps per block 20.5 ms, ten
// 21.7 ms). The single-precision kernel is not fetch-bound: two warps per block, twenty per SM,
// each taking the next pose on its own.
constexpr bool kLockstep = FXE_REFERENCE_FORMULAS;
constexpr int kVorWarps = kLockstep ? 8 : 2;
// The kernel outgrows the instruction cache: its rarely taken or bulky helpers are called, not
// inlined (double build; measured one by one), and no loop is unrolled — every loop carries
// `#pragma unroll 1` unless it says otherwise (measured on GB300, plain-scale workload: 36.0 ->
// 30.4 ms per launch in double precision, 6.8 -> 4.9 ms in single).
#if FXE_REFERENCE_FORMULAS
#define FXE_COLD __noinline__
#else
#define FXE_COLD
#endif
struct __align__(4 * sizeof(real)) real4 {
    real x, y, z, w;
};
struct real3 {
    real x, y, z;
};
__device__ __forceinline__ real4 make_real4(real x, real y, real z, real w) { return real4{x, y, z, w}; }
__device__ __forceinline__ real4 to_real4(const float4& v) { return real4{(real)v.x, (real)v.y, (real)v.z, (real)v.w}; }

template <typename V>
__device__ __forceinline__ void warp_argmin(V& v, int& i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const V v2 = __shfl_xor_sync(kFull, v, o);
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

// ------------------------------------------------------------------------------------------
// per-warp workspace of one polyhedron
// ------------------------------------------------------------------------------------------
struct VorShared {
    real4 pl[kMaxPlanes];          // plane A.x + D = 0 (A unit normal, D = -plane distance)
    real area[kMaxCand];
    int cidx[kMaxCand];             // Calc index of each contact
    uint8_t cslot[kMaxCand];        // the contact's slot in the atom's candidate list
    real4 vx[kMaxVerts];           // vertex x, y, z, distance to the atom centre
    uchar4 vp[kMaxVerts];           // the vertex's planes (kNone = sphere)
    union {
        struct {
            // (two spare slots: the step that reaches the 200-edge limit writes up to two edges)
            real3 ev[kMaxEdges + 2];   // edge direction
            uchar4 ep[kMaxEdges + 2];   // plane0, plane1, start plane, end plane
            uchar2 es[kMaxEdges + 2];   // start vertex, end vertex
        } e;
        struct {
            uint8_t pt[kMaxFacePts];
            real cosv[kMaxFacePts];
        } f;
    } u;
    uint16_t foff[kMaxCand + 1];
    uint8_t fnp[kMaxCand];
    uint16_t toff[kMaxCand + 1];   // per face: first fan triangle / arc segment in the flat lists
    uint16_t aoff[kMaxCand + 1];
    union {
        real tmp[32];                  // one value per lane, for in-order sums
        uint8_t elist[kMaxEdges + 8];  // the hull edges with an end outside the sphere
    };
#if FXE_FILTER
    float4 plf[kMaxPlanes];        // the planes rounded to single precision, for pre-tests
#endif
    uint8_t flag[kMaxPlanes];
    uint8_t sprev[kMaxCand];       // per face: point 1 before a replayed stale read (kNone: none)
    uint8_t flist[kMaxCand];       // faces whose test point is checked against the other planes
    uint8_t llist[kMaxCand];       // faces of two points (lenses), in face order
    uint32_t cmask[kFaceWords];    // faces with a test point
    uint32_t bad[kFaceWords];      // faces whose test point lies in front of another plane
    int eng[4];
    int epi;
    int nv;
};

__device__ __forceinline__ real dot3(const real4& a, real x, real y, real z) {
    return a.x * x + a.y * y + a.z * z;
}

// solve_3x3 (LIB/Vcontacts.cpp:1384-1414) in FP32.
__device__ FXE_COLD bool solve3(const real4& e0, const real4& e1, const real4& e2, real* pt) {
    const real c00 = e1.y * e2.z - e2.y * e1.z;
    const real c01 = -e1.x * e2.z + e2.x * e1.z;
    const real c02 = e1.x * e2.y - e2.x * e1.y;
    const real c10 = -e0.y * e2.z + e2.y * e0.z;
    const real c11 = e0.x * e2.z - e2.x * e0.z;
    const real c12 = -e0.x * e2.y + e2.x * e0.y;
    const real c20 = e0.y * e1.z - e1.y * e0.z;
    const real c21 = -e0.x * e1.z + e1.x * e0.z;
    const real c22 = e0.x * e1.y - e1.x * e0.y;
    const real det = e0.x * c00 + e0.y * c01 + e0.z * c02;
    if (det == real(0.0)) return false;
    pt[0] = -(e0.w * c00 + e1.w * c10 + e2.w * c20) / det;
    pt[1] = -(e0.w * c01 + e1.w * c11 + e2.w * c21) / det;
    pt[2] = -(e0.w * c02 + e1.w * c12 + e2.w * c22) / det;
    return true;
}

// Coordinate i (0..2) of solve3's solution, with the same operations in the same order: each
// lane of a warp can take one coordinate with one instruction stream (the cofactors of column i
// as P*Q - R*S on operands chosen per lane; -a*b + c*d is that value exactly). 0 when det is 0.
__device__ __forceinline__ real solve3_coord(const real4& e0, const real4& e1, const real4& e2, int i) {
    const real c00 = e1.y * e2.z - e2.y * e1.z;
    const real c01 = -e1.x * e2.z + e2.x * e1.z;
    const real c02 = e1.x * e2.y - e2.x * e1.y;
    const real det = e0.x * c00 + e0.y * c01 + e0.z * c02;
    // column i of the cofactors of rows 1 and 2
    const real p1 = i == 0 ? e2.y : i == 1 ? e0.x : e2.x, q1 = i == 0 ? e0.z : i == 1 ? e2.z : e0.y;
    const real r1 = i == 0 ? e0.y : i == 1 ? e2.x : e0.x, s1 = i == 0 ? e2.z : i == 1 ? e0.z : e2.y;
    const real p2 = i == 0 ? e0.y : i == 1 ? e1.x : e0.x, q2 = i == 0 ? e1.z : i == 1 ? e0.z : e1.y;
    const real r2 = i == 0 ? e1.y : i == 1 ? e0.x : e1.x, s2 = i == 0 ? e0.z : i == 1 ? e1.z : e0.y;
    const real c0i = i == 0 ? c00 : i == 1 ? c01 : c02;
    const real c1i = p1 * q1 - r1 * s1;
    const real c2i = p2 * q2 - r2 * s2;
    if (det == real(0.0)) return real(0.0);
    return -(e0.w * c0i + e1.w * c1i + e2.w * c2i) / det;
}

// solve_2xS (LIB/Vcontacts.cpp:1427-1476) in FP32.
// rr is the square of the radius as the reference forms it: a single-precision product.
__device__ FXE_COLD bool solve2s(const real4& a, const real4& b, real rr, real* p0, real* p1) {
    const real e2x = a.y * b.z - a.z * b.y;
    const real e2y = a.z * b.x - a.x * b.z;
    const real e2z = a.x * b.y - a.y * b.x;
    const real c00 = b.y * e2z - e2y * b.z;
    const real c01 = -b.x * e2z + e2x * b.z;
    const real c02 = b.x * e2y - e2x * b.y;
    const real c10 = -a.y * e2z + e2y * a.z;
    const real c11 = a.x * e2z - e2x * a.z;
    const real c12 = -a.x * e2y + e2x * a.y;
    const real det = e2x * e2x + e2y * e2y + e2z * e2z;
    if (det == real(0.0)) return false;
    const real ax = -(a.w * c00 + b.w * c10) / det;
    const real ay = -(a.w * c01 + b.w * c11) / det;
    const real az = -(a.w * c02 + b.w * c12) / det;
    real t = (rr - ax * ax - ay * ay - az * az) / det;
    if (t < real(0.0)) return false;
    t = sqrt(t);
    p0[0] = ax + t * e2x; p0[1] = ay + t * e2y; p0[2] = az + t * e2z;
    p1[0] = ax - t * e2x; p1[1] = ay - t * e2y; p1[2] = az - t * e2z;
    return true;
}

__device__ __forceinline__ real cos_pqr(const real4& p, const real4& q, const real4& r) {
    const real ax = p.x - q.x, ay = p.y - q.y, az = p.z - q.z;
    const real bx = r.x - q.x, by = r.y - q.y, bz = r.z - q.z;
    return (ax * bx + ay * by + az * bz) / sqrt((ax * ax + ay * ay + az * az) * (bx * bx + by * by + bz * bz));
}

// Solid angle at the atom centre of the triangle P0 P1 P2 (Van Oosterom & Strackee,
// IEEE Trans. Biomed. Eng. 30:125, 1983): tan(E/2) = |P0.(P1 x P2)| /
// (|P0||P1||P2| + (P0.P1)|P2| + (P0.P2)|P1| + (P1.P2)|P0|), with the triple product taken on
// the edge vectors P1-P0, P2-P0 so that small triangles keep their precision in FP32.
// .w of each point holds its distance to the centre.
__device__ __forceinline__ real solid_angle(const real4& p0, const real4& p1, const real4& p2) {
    const real ux = p1.x - p0.x, uy = p1.y - p0.y, uz = p1.z - p0.z;
    const real vx = p2.x - p0.x, vy = p2.y - p0.y, vz = p2.z - p0.z;
    const real num = fabs(p0.x * (uy * vz - uz * vy) + p0.y * (uz * vx - ux * vz) + p0.z * (ux * vy - uy * vx));
    const real d01 = p0.x * p1.x + p0.y * p1.y + p0.z * p1.z;
    const real d02 = p0.x * p2.x + p0.y * p2.y + p0.z * p2.z;
    const real d12 = p1.x * p2.x + p1.y * p2.y + p1.z * p2.z;
    const real den = p0.w * p1.w * p2.w + d01 * p2.w + d02 * p1.w + d12 * p0.w;
    return real(2.0) * atan2(num, den);
}

// spherical_arc (LIB/Vcontacts.cpp:1518-1557): the cap sector between B and C about the
// contact centre Ao (the angle B-Ao-C times r (r - h)) minus a spherical triangle. The
// reference's triangle has two sides equal to the angle Ao-O-B and the third equal to B-O-C
// (it assumes C lies on the contact circle too, which projected vertices need not), and its
// half-angle products take absolute values, so the excess it returns is
//   E = 4 atan(|tan(phi/4)| sqrt(|tan((2 theta + phi)/4) tan((2 theta - phi)/4)|))
// with theta = Ao-O-B and phi = B-O-C. The angles come from atan2 of cross and dot products,
// which keeps the result accurate in FP32 when B and C are close.
__device__ __forceinline__ real angle_between(real ux, real uy, real uz, real vx, real vy, real vz) {
    const real wx = uy * vz - uz * vy, wy = uz * vx - ux * vz, wz = ux * vy - uy * vx;
    return atan2(sqrt(wx * wx + wy * wy + wz * wz), ux * vx + uy * vy + uz * vz);
}

#if FXE_REFERENCE_FORMULAS
// The reference's own expression (double builds): reproduces its values, including those of
// nearly degenerate triangles, to rounding.
__device__ FXE_COLD real sph_arc(const real4& ao, const real4& b, const real4& c, real rado) {
    const real cosAOB = (ao.x * b.x + ao.y * b.y + ao.z * b.z) / (ao.w * b.w);
    const real cosBOC = (b.x * c.x + b.y * c.y + b.z * c.z) / (b.w * c.w);
    // (x / 8 and x * 0.125 are the same correctly rounded value: the multiply is the cheaper)
    const real h = sqrt((1 + cosBOC) * real(0.125));
    const real U = (1 + cosAOB) * h;
    const real V = (1 - cosAOB) * h;
    const real W = sqrt((1 - cosAOB) * (1 + cosAOB) * (1 - cosBOC) * real(0.125));
    const real tS = (1 - U + V + W + W) / (1 + U - V - W - W);
    const real tSB = (1 - U - V) / (1 + U + V);
    const real tSA = (1 - U + V - W - W) / (1 + U - V + W + W);
    real tanprod = real(0.0);
    if ((tS * tSA) > real(0.0)) tanprod = sqrt(tSB * tSB * tS * tSA);
    const real px = b.x - ao.x, py = b.y - ao.y, pz = b.z - ao.z;
    const real qx = c.x - ao.x, qy = c.y - ao.y, qz = c.z - ao.z;
    const real cosBAC = (px * qx + py * qy + pz * qz) / sqrt((px * px + py * py + pz * pz) * (qx * qx + qy * qy + qz * qz));
    real angBAC;
    if (cosBAC > real(1.0)) angBAC = real(0.0);
    else if (cosBAC < real(-1.0)) angBAC = (real)kPi;
    else angBAC = acos(cosBAC);
    return rado * (angBAC * (rado - ao.w) - real(4.0) * rado * atan(sqrt(tanprod)));
}
#else
__device__ FXE_COLD real sph_arc(const real4& ao, const real4& b, const real4& c, real rado) {
    const real sector = angle_between(b.x - ao.x, b.y - ao.y, b.z - ao.z, c.x - ao.x, c.y - ao.y, c.z - ao.z);
    const real th = angle_between(ao.x, ao.y, ao.z, b.x, b.y, b.z);
    const real ph = angle_between(b.x, b.y, b.z, c.x, c.y, c.z);
    const real t = fabs(tan((real(2.0) * th + ph) * real(0.25)) * tan((real(2.0) * th - ph) * real(0.25)));
    const real tri = real(4.0) * atan(fabs(tan(ph * real(0.25))) * sqrt(t));
    return rado * (sector * (rado - ao.w) - rado * tri);
}
#endif

__device__ __forceinline__ real4 centre_of(const real4& pl) {
    return make_real4(-pl.x * pl.w, -pl.y * pl.w, -pl.z * pl.w, fabs(pl.w));
}

// test_point (LIB/Vcontacts.cpp:1357-1372) for several faces at once: face X of sh.flist[0, nf) keeps its test point, held in
// sh.u.f.cosv[3X .. 3X+2], when the point lies behind every flagged contact plane other than X.
// The (face, plane) pairs are spread over the lanes; a face with a plane in front of its point
// gets its bit in sh.bad.
__device__ void faces_inside(VorShared& sh, int NC, int nf, int lane) {
    if (lane < kFaceWords) sh.bad[lane] = 0u;
    __syncwarp();
    const int n = nf * NC;
    #pragma unroll 1
    for (int k = lane; k < n; k += 32) {
        const int fi = k / NC, cp = k - fi * NC;
        const int X = sh.flist[fi];
        if (cp == X || sh.flag[cp] == 0) continue;
        const real* q = &sh.u.f.cosv[3 * X];
        if (dot3(sh.pl[cp], q[0], q[1], q[2]) + sh.pl[cp].w > real(0.0)) atomicOr(&sh.bad[X >> 5], 1u << (X & 31));
    }
    __syncwarp();
}

// add_vedge (LIB/Vcontacts.cpp:633-660): edge en along planes p0 and p1 from vertex sp (at s),
// pointing away from plane tp.
__device__ void add_edge(VorShared& sh, int en, int p0, int p1, int tp, int sp, const real* s) {
    const real4 a = sh.pl[p0], b = sh.pl[p1];
    real vx = a.y * b.z - a.z * b.y;
    real vy = a.z * b.x - a.x * b.z;
    real vz = a.x * b.y - a.y * b.x;
    const real4 t = sh.pl[tp];
    const real tv = t.x * (s[0] + vx) + t.y * (s[1] + vy) + t.z * (s[2] + vz) + t.w;
    if (tv > real(0.0)) { vx = -vx; vy = -vy; vz = -vz; }
    sh.u.e.ev[en] = real3{vx, vy, vz};
    sh.u.e.ep[en] = make_uchar4((uint8_t)p0, (uint8_t)p1, (uint8_t)tp, kNone);
    sh.u.e.es[en] = make_uchar2((uint8_t)sp, kNone);
}

struct WalkStep {
    real x, y, z;
    int pc;      // closing plane, -1 if none
};

#if FXE_FILTER
// Single-precision value of vt = -(P.s + w) / (P.V) and a bound on its distance from the same
// expression evaluated in double: every input is rounded once to float and every operation
// rounds, 16 units of roundoff (2^-20) per sum of absolute terms covers both; the quotients use
// the fast reciprocal (at most 2 units in the last place off, covered by 4 units of |vt| and the
// 1/16 margin on the bound). den_ok is false when the sign of P.V is not certain (the double test
// skips P.V == 0 exactly), when |P.V| is too small for the fast quotient, or when the bound is
// not finite.
__device__ __forceinline__ float vt_pretest(const float4& P, float sx, float sy, float sz, float Vx,
                                            float Vy, float Vz, float* err, bool* den_ok) {
    const float g = 9.5367431640625e-07f;   // 2^-20
    const float den = P.x * Vx + P.y * Vy + P.z * Vz;
    const float eden = g * (fabsf(P.x * Vx) + fabsf(P.y * Vy) + fabsf(P.z * Vz));
    const float num = P.x * sx + P.y * sy + P.z * sz + P.w;
    const float enm = g * (fabsf(P.x * sx) + fabsf(P.y * sy) + fabsf(P.z * sz) + fabsf(P.w));
    // an all-zero normal (an excluded candidate's inert plane) has P.V == 0 exactly in double
    // too, and the double test skips it; report it as a decided non-positive value
    if (P.x == 0.0f && P.y == 0.0f && P.z == 0.0f) {
        *den_ok = true;
        *err = 0.0f;
        return -1.0f;
    }
    const bool ok = fabsf(den) > 2.0f * eden && fabsf(den) > 1e-30f;
    const float vt = __fdividef(-num, den);
    const float er = __fdividef(enm + fabsf(vt) * eden, fabsf(den) - eden) * 1.0625f + fabsf(vt) * 4.8e-7f;
    *den_ok = ok && er < 3.0e38f;
    *err = er;
    return vt;
}
#endif

// The vertex that ends edge e (LIB/Vcontacts.cpp:283-330), in full precision: the plane with
// the smallest positive vt along the edge (planes spread over the lanes) and, when that point
// lies outside the sphere, the bounding planes too. The result is uniform across the warp.
__device__ FXE_COLD WalkStep walk_step_exact(const VorShared& sh, int NC, int e, real rr, int lane) {
    const uchar4 ep = sh.u.e.ep[e];
    const real3 V = sh.u.e.ev[e];
    const real4 s = sh.vx[sh.u.e.es[e].x];
    const int pA = ep.x, pB = ep.y, oldC = ep.z;
    real vtmin = real(9.9e9);
    int pC = INT_MAX;
    #pragma unroll 1
    for (int c = lane; c < NC; c += 32) {
        if (c == pA || c == pB || c == oldC) continue;
        const real4 P = sh.pl[c];
        const real den = P.x * V.x + P.y * V.y + P.z * V.z;
        if (den != real(0.0)) {
            const real vt = -(P.x * s.x + P.y * s.y + P.z * s.z + P.w) / den;
            if (vt < vtmin && vt > real(0.0)) { vtmin = vt; pC = c; }
        }
    }
    warp_argmin(vtmin, pC);
    real x = s.x + vtmin * V.x, y = s.y + vtmin * V.y, z = s.z + vtmin * V.z;
    if (x * x + y * y + z * z > rr) {
        real bvt = vtmin;
        int bc = pC;
        if (lane < 4) {
            const int c = NC + lane;
            if (c != pA && c != pB && c != oldC) {
                const real4 P = sh.pl[c];
                const real den = P.x * V.x + P.y * V.y + P.z * V.z;
                if (den != real(0.0)) {
                    const real vt = -(P.x * s.x + P.y * s.y + P.z * s.z + P.w) / den;
                    if (vt < bvt && vt > real(0.0)) { bvt = vt; bc = c; }
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
    WalkStep r;
    r.x = x;
    r.y = y;
    r.z = z;
    r.pc = pC == INT_MAX ? -1 : pC;
    return r;
}

// The hull walk steps several open edges at once: a step's result depends only on its edge (start
// vertex, direction, planes), all fixed when the edge was made, and the reference takes every edge
// that is open now, in index order, before any edge the steps append (those get higher indices).
// So the first kWalkGroups open edges are stepped together, one group of kWalkLanes lanes each (the
// double-precision arithmetic of the step then serves four edges per warp instruction), and their
// results are booked one after another in index order, skipping an edge an earlier one closed.
constexpr int kWalkGroups = 4;
constexpr int kWalkLanes = 32 / kWalkGroups;

struct GroupStep {
    real x, y, z;
    int pc;        // closing plane, -1 if none
    bool unsure;   // the single-precision pre-tests did not decide it: redo with walk_step_exact
};

// Argmin over the lanes of one group (ties to the lower plane index, as the reference's strict
// less-than over planes in index order keeps the first).
template <typename V>
__device__ __forceinline__ void group_argmin(V& v, int& i) {
#pragma unroll
    for (int o = kWalkLanes / 2; o > 0; o >>= 1) {
        const V v2 = __shfl_xor_sync(kFull, v, o);
        const int i2 = __shfl_xor_sync(kFull, i, o);
        if (v2 < v || (v2 == v && i2 < i)) {
            v = v2;
            i = i2;
        }
    }
}

// One step for the group's edge e (e < 0: the group idles; every lane still joins the shuffles).
// sub: the lane's index in its group; gmask: the group's lanes.
__device__ GroupStep walk_step_group(const VorShared& sh, int NC, int e, real rr, int sub, unsigned gmask) {
    const bool has = e >= 0;
    uchar4 ep = make_uchar4(kNone, kNone, kNone, kNone);
    real3 V = real3{real(0.0), real(0.0), real(0.0)};
    real4 s = make_real4(real(0.0), real(0.0), real(0.0), real(0.0));
    if (has) {
        ep = sh.u.e.ep[e];
        V = sh.u.e.ev[e];
        s = sh.vx[sh.u.e.es[e].x];
    }
    const int pA = ep.x, pB = ep.y, oldC = ep.z;
    GroupStep r;
#if FXE_FILTER
    // planes pre-tested in single precision; when the winner is surely positive and every other
    // plane surely not positive or surely farther, only the winner's vt is evaluated in double
    const float sx = (float)s.x, sy = (float)s.y, sz = (float)s.z;
    const float Vx = (float)V.x, Vy = (float)V.y, Vz = (float)V.z;
    float best = 9.9e9f, beste = 0.0f;
    int bi = INT_MAX;
    // and the two smallest lower bounds (vt - err) over the planes whose vt may be positive: every
    // plane but the winner must be surely not positive or surely farther
    float lo1 = 3.0e38f, lo2 = 3.0e38f;
    int lo1i = INT_MAX;
    bool unsure = false;
    if (has) {
        #pragma unroll 1
        for (int c = sub; c < NC; c += kWalkLanes) {
            if (c == pA || c == pB || c == oldC) continue;
            float er;
            bool ok;
            const float vt = vt_pretest(sh.plf[c], sx, sy, sz, Vx, Vy, Vz, &er, &ok);
            if (!ok) {
                unsure = true;
                continue;
            }
            if (vt > 0.0f && vt < best) { best = vt; beste = er; bi = c; }
            if (vt + er > 0.0f) {
                const float lo = vt - er;
                if (lo < lo1) { lo2 = lo1; lo1 = lo; lo1i = c; }
                else if (lo < lo2) lo2 = lo;
            }
        }
    }
#pragma unroll
    for (int o = kWalkLanes / 2; o > 0; o >>= 1) {
        const float b2 = __shfl_xor_sync(kFull, best, o);
        const float e2 = __shfl_xor_sync(kFull, beste, o);
        const int i2 = __shfl_xor_sync(kFull, bi, o);
        if (b2 < best || (b2 == best && i2 < bi)) { best = b2; beste = e2; bi = i2; }
    }
    if (bi != INT_MAX && !(best - beste > 0.0f)) unsure = true;
    const float mylo = lo1i == bi ? lo2 : lo1;
    if (mylo < 3.0e38f && !(bi != INT_MAX && mylo > best + beste)) unsure = true;
    unsure = (__ballot_sync(kFull, unsure) & gmask) != 0u;
    real vtmin = real(9.9e9);
    if (!unsure && bi != INT_MAX) {
        const real4 P = sh.pl[bi];
        const real den = P.x * V.x + P.y * V.y + P.z * V.z;
        vtmin = -(P.x * s.x + P.y * s.y + P.z * s.z + P.w) / den;
    }
    r.x = s.x + vtmin * V.x;
    r.y = s.y + vtmin * V.y;
    r.z = s.z + vtmin * V.z;
    // outside the sphere: the bounding planes (10 A out) are most of the time surely farther
    bool need = false;
    if (has && !unsure && r.x * r.x + r.y * r.y + r.z * r.z > rr) {
        need = bi == INT_MAX;
        if (!need && sub < 4) {
            const int c = NC + sub;
            if (c != pA && c != pB && c != oldC) {
                float er;
                bool ok;
                const float vt = vt_pretest(sh.plf[c], sx, sy, sz, Vx, Vy, Vz, &er, &ok);
                need = !(ok && (vt + er <= 0.0f || vt - er > (float)vtmin * 1.0000005f));
            }
        }
    }
    // (every lane takes part in the ballot: it must not sit behind a short-circuit)
    const unsigned need_lanes = __ballot_sync(kFull, need);
    r.unsure = unsure || (need_lanes & gmask) != 0u;
    r.pc = bi == INT_MAX ? -1 : bi;
#else
    real vtmin = real(9.9e9);
    int pC = INT_MAX;
    if (has) {
        #pragma unroll 1
        for (int c = sub; c < NC; c += kWalkLanes) {
            if (c == pA || c == pB || c == oldC) continue;
            const real4 P = sh.pl[c];
            const real den = P.x * V.x + P.y * V.y + P.z * V.z;
            if (den != real(0.0)) {
                const real vt = -(P.x * s.x + P.y * s.y + P.z * s.z + P.w) / den;
                if (vt < vtmin && vt > real(0.0)) { vtmin = vt; pC = c; }
            }
        }
    }
    group_argmin(vtmin, pC);
    r.x = s.x + vtmin * V.x;
    r.y = s.y + vtmin * V.y;
    r.z = s.z + vtmin * V.z;
    const bool out = has && r.x * r.x + r.y * r.y + r.z * r.z > rr;
    if (out && sub < 4) {
        const int c = NC + sub;
        if (c != pA && c != pB && c != oldC) {
            const real4 P = sh.pl[c];
            const real den = P.x * V.x + P.y * V.y + P.z * V.z;
            if (den != real(0.0)) {
                const real vt = -(P.x * s.x + P.y * s.y + P.z * s.z + P.w) / den;
                if (vt < vtmin && vt > real(0.0)) { vtmin = vt; pC = c; }
            }
        }
    }
    group_argmin(vtmin, pC);
    if (out) {
        r.x = s.x + vtmin * V.x;
        r.y = s.y + vtmin * V.y;
        r.z = s.z + vtmin * V.z;
    }
    r.pc = pC == INT_MAX ? -1 : pC;
    r.unsure = false;
#endif
    return r;
}

// Face of flat item k: the last face X in [0, NC) whose first item is at or before k.
__device__ __forceinline__ int face_of(const uint16_t* off, int NC, int k) {
    int lo = 0, hi = NC;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((int)off[mid] <= k) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Whether points vi and vi+1 of a face bound an arc segment: both arc points, of different
// edges (LIB/Vcontacts.cpp:943-954).
__device__ __forceinline__ int arc_segment(const VorShared& sh, const uint8_t* pt, int np, int vi) {
    const uchar4 qa = sh.vp[pt[vi]], qb = sh.vp[pt[(vi + 1) % np]];
    if (qa.z != kNone || qb.z != kNone) return 0;
    const int sa = (qa.y == kNone ? -1 : qa.y) + qa.x;
    const int sb = (qb.y == kNone ? -1 : qb.y) + qb.x;
    return sa != sb;
}

// Area of the fan triangle v0 va vb on the sphere of radius rado.
__device__ __forceinline__ real fan_triangle(const real4& v0, const real4& va, const real4& vb, real rado) {
#if FXE_REFERENCE_FORMULAS
    // L'Huilier-type tangent products as the reference writes them (LIB/Vcontacts.cpp:927-940)
    const real cNN1 = (va.x * vb.x + va.y * vb.y + va.z * vb.z) / (va.w * vb.w);
    const real cN0a = (v0.x * va.x + v0.y * va.y + v0.z * va.z) / (v0.w * va.w);
    const real cN0b = (v0.x * vb.x + v0.y * vb.y + v0.z * vb.z) / (v0.w * vb.w);
    // (x / 8 and x * 0.125 are the same correctly rounded value: the multiply is the cheaper)
    const real U = sqrt((1 + cN0a) * (1 + cNN1) * (1 + cN0b) * real(0.125));
    const real V = sqrt((1 - cN0a) * (1 - cNN1) * (1 + cN0b) * real(0.125));
    const real W = sqrt((1 - cN0a) * (1 + cNN1) * (1 - cN0b) * real(0.125));
    const real Xv = sqrt((1 + cN0a) * (1 - cNN1) * (1 - cN0b) * real(0.125));
    const real tS = (1 - U + V + W + Xv) / (1 + U - V - W - Xv);
    const real tSA = (1 - U - V - W + Xv) / (1 + U + V + W - Xv);
    const real tSB = (1 - U - V + W - Xv) / (1 + U + V - W + Xv);
    const real tSC = (1 - U + V - W - Xv) / (1 + U - V + W + Xv);
    const real tanprod = sqrt(tS * tSA * tSB * tSC);
    return tanprod > real(0.0) ? real(4.0) * rado * rado * atan(sqrt(tanprod)) : real(0.0);
#else
    // the same triangle's solid angle, well conditioned in FP32
    return rado * rado * solid_angle(v0, va, vb);
#endif
}

// Adds each lane's value v to the area of face X (X < 0: nothing), lanes of one face in lane
// order, so that a face's sum is formed in the order of its items.
__device__ __forceinline__ void add_in_order(VorShared& sh, int X, real v, int lane) {
    sh.tmp[lane] = v;
    const unsigned grp = __match_any_sync(kFull, X);
    __syncwarp();
    if (X >= 0 && lane == __ffs(grp) - 1) {
        real acc = sh.area[X];
        #pragma unroll 1
        for (unsigned m = grp; m; m &= m - 1) acc += sh.tmp[__ffs(m) - 1];
        sh.area[X] = acc;
    }
    __syncwarp();
}

// The face that the arc between points cur and nxt of engulfed face X is credited to
// (LIB/Vcontacts.cpp:971-1000): the plane the two points share besides X, when it is neither the
// sphere nor an engulfing plane; -1 when the reference moves on without crediting anything.
__device__ __forceinline__ int engulf_comm(const VorShared& sh, int NC, int X, int cur, int nxt) {
    const uchar4 qc = sh.vp[cur], qn = sh.vp[nxt];
    int pa1, pa2;
    if (qc.x == X) { pa1 = qc.y; pa2 = qc.z; }
    else { pa1 = qc.x; pa2 = (qc.y == X) ? qc.z : qc.y; }
    int comm;
    if (pa1 == qn.x || pa1 == qn.y || pa1 == qn.z) comm = pa1;
    else if (pa2 == qn.x || pa2 == qn.y || pa2 == qn.z) comm = pa2;
    else return -1;
    return (comm != kNone && !(comm < NC && (sh.flag[comm] & kEngulf))) ? comm : -1;
}

// Corrections for engulfing planes (LIB/Vcontacts.cpp:963-1041): arcs of the engulfed faces
// credited to their neighbours, then the engulfing faces' own areas. The reference walks the
// engulfed faces' points one after another; here each (face, point) item of the flat face lists
// goes to a lane, the arcs are evaluated together, and each neighbour's sum is formed in the
// reference's order. tot_pts: the length of the flat face lists.
__device__ FXE_COLD void engulf_corrections(VorShared& sh, int NC, int tot_pts, real rado, real rr, real two_pi_r,
                                            int epi, int lane) {
    if (epi > 0) {
        // the items that credit an arc, in order, packed (face, current point, next point,
        // neighbour) into the cosine scratch (free by now), then their arcs a warp at a time
        uint32_t* items = reinterpret_cast<uint32_t*>(sh.u.f.cosv);
        int n_items = 0;
        #pragma unroll 1
        for (int k0 = 0; k0 < tot_pts; k0 += 32) {
            const int k = k0 + lane;
            int comm = -1, X = 0, cur = 0, nxt = 0;
            if (k < tot_pts) {
                X = face_of(sh.foff, NC, k);
                const int vi = k - sh.foff[X];
                const int np = sh.fnp[X];
                if ((sh.flag[X] & kEngulf) && vi < np) {
                    const uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
                    // a face of two points stops after its first credited (or sphere-bound) arc
                    if (!(np == 2 && vi == 1 && engulf_comm(sh, NC, X, pt[0], pt[1]) >= 0)) {
                        cur = pt[vi];
                        nxt = pt[(vi + 1) % np];
                        const int c = engulf_comm(sh, NC, X, cur, nxt);
                        if (c >= 0 && c < NC) comm = c;
                    }
                }
            }
            const unsigned m = __ballot_sync(kFull, comm >= 0);
            if (comm >= 0)
                items[n_items + __popc(m & lanemask_lt())] =
                    (uint32_t)X | ((uint32_t)cur << 8) | ((uint32_t)nxt << 16) | ((uint32_t)comm << 24);
            n_items += __popc(m);
        }
        __syncwarp();
        // two engulfing planes: the lens their circles cut, its two arcs evaluated with the items
        // (the last two of the list)
        real q0[3] = {real(0.0), real(0.0), real(0.0)}, q1[3] = {real(0.0), real(0.0), real(0.0)};
        const bool lens2 = epi == 2 && solve2s(sh.pl[sh.eng[0]], sh.pl[sh.eng[1]], rr, q0, q1);
        const int n_all = n_items + (lens2 ? 2 : 0);
        real m = real(0.0);   // lane 0: the sum of the two lens arcs
        #pragma unroll 1
        for (int k0 = 0; k0 < n_all; k0 += 32) {
            const int k = k0 + lane;
            int comm = -1;
            real v = real(0.0);
            if (k < n_all) {
                real4 ao, b, c;
                if (k < n_items) {
                    const uint32_t it = items[k];
                    comm = (int)(it >> 24);
                    ao = centre_of(sh.pl[it & 0xffu]);
                    b = sh.vx[(it >> 8) & 0xffu];
                    c = sh.vx[(it >> 16) & 0xffu];
                } else {
                    ao = centre_of(sh.pl[sh.eng[k - n_items]]);
                    b = make_real4(q0[0], q0[1], q0[2], rado);
                    c = make_real4(q1[0], q1[1], q1[2], rado);
                }
                v = sph_arc(ao, b, c, rado);
            }
            add_in_order(sh, comm, v, lane);
            if (lens2) {
                // the reference adds the second arc to the first
                const real a0 = __shfl_sync(kFull, v, n_items & 31);
                const real a1 = __shfl_sync(kFull, v, (n_items + 1) & 31);
                if (lane == 0) {
                    if (k0 <= n_items && n_items < k0 + 32) m = a0;
                    if (k0 <= n_items + 1 && n_items + 1 < k0 + 32) m += a1;
                }
            }
        }
        if (epi == 1) {
            if (lane == 0) sh.area[sh.eng[0]] = two_pi_r * (rado + fabs(sh.pl[sh.eng[0]].w));
        } else if (epi == 2 && lane == 0) {
            const real full = two_pi_r * rado;
            if (!lens2) {
                sh.area[sh.eng[0]] = full;
                sh.area[sh.eng[1]] = full;
            } else {
                sh.area[sh.eng[0]] = full - real(0.5) * m;
                sh.area[sh.eng[1]] = full - real(0.5) * m;
            }
        }
        __syncwarp();
        if (epi >= 3) {
            const real share = real(4.0) * (real)kPi * rado * rado / epi;
            #pragma unroll 1
            for (int X = lane; X < NC; X += 32) sh.area[X] = (sh.flag[X] & kEngulf) ? share : real(0.0);
        }
        __syncwarp();
    }
}

// Face history of one pose (reference face order): order_faces leaves each contact's point list
// in ptorder[X].pt[] (LIB/Vcontacts.cpp:726-831), a workspace that outlives the atom, and reads
// ptorder[X].pt[numpts] — a slot past the face's own list — when no point shares the first
// point's second plane (:800-812). That slot holds what an earlier atom of the pose left there
// (zero at the start of the pose). The history keeps those lists per contact index X, rows of
// kHistPts entries, followed by the pre-extra contents of the vertex slots the antipodal points
// take (the reference appends them one face at a time, so a face's read of a later face's slot
// still sees the old vertex there).
constexpr int kHistPts = 64;
constexpr int kHistBytes = kMaxCand * kHistPts;
constexpr size_t kHistStride = kHistBytes + kMaxCand * (sizeof(real4) + sizeof(uchar4));
static_assert(kHistBytes % 32 == 0 && kHistStride % 32 == 0, "history rows keep 32-byte alignment");

__device__ __forceinline__ real4* hist_vx(uint8_t* h) { return reinterpret_cast<real4*>(h + kHistBytes); }
__device__ __forceinline__ uchar4* hist_vp(uint8_t* h) {
    return reinterpret_cast<uchar4*>(h + kHistBytes + kMaxCand * sizeof(real4));
}

// One extended-radical-plane polyhedron and its contact areas. sh.pl/flag/cidx hold the
// planes of the NC contacts in the order of the reference's contact list. hist: the pose's face
// history (reference face order), or null (a face whose first point has no neighbour on its
// second plane is then ordered from the point's other plane). Returns kAtomOk, kAtomHullFail
// (the walk reached 200 edges) or kAtomCapacity.
__device__ int voronoi_warp(VorShared& sh, int NC, real rado, int lane, int* no_partner, int* unreplayed,
                            int seedA, int seedB, int seedC, uint8_t* hist) {
    // rado * rado in single precision, as the reference squares its float radius
    const real rr = (real)((float)rado * (float)rado);
    // bounding planes
    if (lane < 4) {
        const real bx[4] = {real(0.707), real(0.707), -real(0.707), -real(0.707)};
        const real by[4] = {real(1.0), -real(1.0), real(0.0), real(0.0)};
        const real bz[4] = {real(0.0), real(0.0), real(1.0), -real(1.0)};
        sh.pl[NC + lane] = make_real4(bx[lane], by[lane], bz[lane], -real(10.0));
#if FXE_FILTER
        sh.plf[NC + lane] = make_float4((float)bx[lane], (float)by[lane], (float)bz[lane], -10.0f);
#endif
        sh.flag[NC + lane] = 0;
    }
    #pragma unroll 1
    for (int c = lane; c < NC; c += 32) sh.area[c] = real(0.0);
    __syncwarp();

    // ---- first vertex: the seed left by an earlier atom, else get_firstvert's search from the
    //      plane closest to the centre (LIB/Vcontacts.cpp:498-592) ----
    int pA0, pB0, pC0;
    if (seedA >= 0 && seedB >= 0 && seedC >= 0) {
        pA0 = seedA;
        pB0 = seedB;
        pC0 = seedC;
    } else {
    real bv = real(9.9e9);
    int bi = INT_MAX;
    #pragma unroll 1
    for (int c = lane; c < NC; c += 32) {
        const real d = fabs(sh.pl[c].w);
        if (d < bv) { bv = d; bi = c; }
    }
    warp_argmin(bv, bi);
    pA0 = bi;
    if (pA0 == INT_MAX) return kAtomCapacity;
    const real4 A = sh.pl[pA0];
    bv = real(9.9e9);
    bi = INT_MAX;
    #pragma unroll 1
    for (int c = lane; c < NC + 4; c += 32) {
        if (c == pA0) continue;
        const real4 C = sh.pl[c];
        const real4 v = make_real4(A.y * C.z - A.z * C.y, A.z * C.x - A.x * C.z, A.x * C.y - A.y * C.x, real(0.0));
        real t[3];
        if (solve3(A, C, v, t)) {
            const real d = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
            if (d < bv) { bv = d; bi = c; }
        }
    }
    warp_argmin(bv, bi);
    pB0 = bi;
    if (pB0 == INT_MAX) return kAtomCapacity;
    const real4 B = sh.pl[pB0];
    const real4 v = make_real4(A.y * B.z - A.z * B.y, A.z * B.x - A.x * B.z, A.x * B.y - A.y * B.x, real(0.0));
    real ptA[3];
    solve3(A, B, v, ptA);
    bv = real(9.9e9);
    bi = INT_MAX;
    #pragma unroll 1
    for (int c = lane; c < NC + 4; c += 32) {
        if (c == pA0 || c == pB0) continue;
        const real4 C = sh.pl[c];
        const real den = C.x * v.x + C.y * v.y + C.z * v.z;
        if (den != real(0.0)) {
            const real vt = fabs(-(C.x * ptA[0] + C.y * ptA[1] + C.z * ptA[2] + C.w) / den);
            if (vt < bv) { bv = vt; bi = c; }
        }
    }
    warp_argmin(bv, bi);
    pC0 = bi;
    if (pC0 == INT_MAX) return kAtomCapacity;
    }
    {
        // the vertex's coordinates on lanes 0..2, then its three edges at once
        const real ti = solve3_coord(sh.pl[pA0], sh.pl[pB0], sh.pl[pC0], lane < 3 ? lane : 0);
        real t[3];
        t[0] = __shfl_sync(kFull, ti, 0);
        t[1] = __shfl_sync(kFull, ti, 1);
        t[2] = __shfl_sync(kFull, ti, 2);
        if (lane == 0) {
            sh.vx[0] = make_real4(t[0], t[1], t[2], real(0.0));   // (its distance comes with the others')
            sh.vp[0] = make_uchar4((uint8_t)pA0, (uint8_t)pB0, (uint8_t)pC0, 0);
            sh.flag[pA0] |= kOnHull;
            sh.flag[pB0] |= kOnHull;
            sh.flag[pC0] |= kOnHull;
        }
        if (lane < 3) {
            const int p0 = lane == 0 ? pA0 : lane == 1 ? pB0 : pC0;
            const int p1 = lane == 0 ? pB0 : lane == 1 ? pC0 : pA0;
            const int tp = lane == 0 ? pC0 : lane == 1 ? pA0 : pB0;
            add_edge(sh, lane, p0, p1, tp, 0, t);
        }
    }
    __syncwarp();

    // ---- hull walk (LIB/Vcontacts.cpp:262-410), the open edges stepped kWalkGroups at a time ----
    int edgenum = 3, startedge = 0, vn = 1;
    const int sub = lane & (kWalkLanes - 1);
    const unsigned gmask = ((1u << kWalkLanes) - 1u) << (lane & ~(kWalkLanes - 1));
    #pragma unroll 1
    for (;;) {
        while (startedge < edgenum && sh.u.e.es[startedge].y != kNone) ++startedge;
        if (startedge >= edgenum) break;
        // the first kWalkGroups open edges, in index order (one byte each)
        unsigned batch = 0u;
        int nb = 0;
        #pragma unroll 1
        for (int e0 = startedge; e0 < edgenum && nb < kWalkGroups; e0 += 32) {
            const int f = e0 + lane;
            unsigned m = __ballot_sync(kFull, f < edgenum && sh.u.e.es[f].y == kNone);
            while (m && nb < kWalkGroups) {
                batch |= (unsigned)(e0 + __ffs(m) - 1) << (8 * nb);
                m &= m - 1;
                ++nb;
            }
        }
        const int grp = lane / kWalkLanes;
        const GroupStep gs = walk_step_group(sh, NC, grp < nb ? (int)((batch >> (8 * grp)) & 0xffu) : -1, rr, sub, gmask);
        // book the steps in index order; a new vertex's coordinates are stored by its group's
        // first lane and a new edge's direction is set after the batch (lane j holds the j-th new
        // edge: slot, planes, start vertex)
        real gx = gs.x, gy = gs.y, gz = gs.z;
        int my_vn = -1;
        int n_pend = 0, pe = 0, p0e = 0, pce = 0, tpe = 0, pve = 0;
        #pragma unroll 1
        for (int g = 0; g < nb; ++g) {
            const int e = (batch >> (8 * g)) & 0xffu;
            const int pu = __shfl_sync(kFull, (gs.pc << 1) | (int)gs.unsure, g * kWalkLanes);
            int pC = pu >> 1;   // (an arithmetic shift keeps -1)
            const bool unsure = (pu & 1) != 0;
            if (sh.u.e.es[e].y != kNone) continue;   // closed by an earlier edge of the batch
            startedge = e;
            if (unsure) {
                const WalkStep w = walk_step_exact(sh, NC, e, rr, lane);
                if (lane == g * kWalkLanes) {
                    gx = w.x;
                    gy = w.y;
                    gz = w.z;
                }
                pC = w.pc;
            }
            if (pC < 0) return kAtomHullFail;
            if (vn >= kMaxVerts - 1) return kAtomCapacity;
            const uchar4 ep = sh.u.e.ep[e];
            const int pA = ep.x, pB = ep.y;
            // edges (pA, pC) and (pB, pC): the first match after this edge, else a new edge
            int mAC = INT_MAX, mBC = INT_MAX;
            #pragma unroll 1
            for (int e0 = e + 1; e0 < edgenum; e0 += 32) {
                const int f = e0 + lane;
                bool ac = false, bc = false;
                if (f < edgenum) {
                    const uchar4 q = sh.u.e.ep[f];
                    ac = (q.x == pA && q.y == pC) || (q.x == pC && q.y == pA);
                    bc = (q.x == pB && q.y == pC) || (q.x == pC && q.y == pB);
                }
                const unsigned ma = __ballot_sync(kFull, ac), mb = __ballot_sync(kFull, bc);
                if (ma && mAC == INT_MAX) mAC = e0 + __ffs(ma) - 1;
                if (mb && mBC == INT_MAX) mBC = e0 + __ffs(mb) - 1;
                if (mAC != INT_MAX && mBC != INT_MAX) break;
            }
            __syncwarp();
            // a walk that keeps opening edges past the reference's 200-edge check ends here: as a
            // hull failure when the reference's check fails it at this step, else over capacity
            const int n_new = (mAC == INT_MAX) + (mBC == INT_MAX);
            if (edgenum + n_new > kMaxEdges + 2) return mBC == INT_MAX ? kAtomHullFail : kAtomCapacity;
            const int eAC = mAC != INT_MAX ? mAC : edgenum;
            const int eBC = mBC != INT_MAX ? mBC : edgenum + (mAC == INT_MAX ? 1 : 0);
            if (lane == g * kWalkLanes) my_vn = vn;
            if (lane == 0) {
                sh.vp[vn] = make_uchar4((uint8_t)pA, (uint8_t)pB, (uint8_t)pC, 0);
                sh.u.e.es[e].y = (uint8_t)vn;
                sh.u.e.ep[e].w = (uint8_t)pC;
                sh.flag[pC] |= kOnHull;
            }
            if (lane < 2) {
                const bool match = lane == 0 ? mAC != INT_MAX : mBC != INT_MAX;
                const int ee = lane == 0 ? eAC : eBC;
                const int p0 = lane == 0 ? pA : pB, tp = lane == 0 ? pB : pA;
                if (match) {
                    sh.u.e.es[ee].y = (uint8_t)vn;
                    sh.u.e.ep[ee].w = (uint8_t)tp;
                } else {
                    sh.u.e.ep[ee] = make_uchar4((uint8_t)p0, (uint8_t)pC, (uint8_t)tp, kNone);
                    sh.u.e.es[ee] = make_uchar2((uint8_t)vn, kNone);
                }
            }
            const int jAC = n_pend, jBC = n_pend + (mAC == INT_MAX ? 1 : 0);
            if (mAC == INT_MAX && lane == jAC) { pe = eAC; p0e = pA; pce = pC; tpe = pB; pve = vn; }
            if (mBC == INT_MAX && lane == jBC) { pe = eBC; p0e = pB; pce = pC; tpe = pA; pve = vn; }
            n_pend += n_new;
            if (mAC == INT_MAX) ++edgenum;
            if (mBC == INT_MAX) {
                ++edgenum;
                if (edgenum >= kMaxEdges) return kAtomHullFail;
            }
            ++vn;
            __syncwarp();
        }
        if (my_vn >= 0) sh.vx[my_vn] = make_real4(gx, gy, gz, real(0.0));
        __syncwarp();
        // the new edges' directions, oriented away from their third plane (add_vedge)
        if (lane < n_pend) {
            const real4 a = sh.pl[p0e], b = sh.pl[pce], t = sh.pl[tpe];
            const real4 r = sh.vx[pve];
            real vx = a.y * b.z - a.z * b.y;
            real vy = a.z * b.x - a.x * b.z;
            real vz = a.x * b.y - a.y * b.x;
            const real tv = t.x * (r.x + vx) + t.y * (r.y + vy) + t.z * (r.z + vz) + t.w;
            if (tv > real(0.0)) { vx = -vx; vy = -vy; vz = -vz; }
            sh.u.e.ev[pe] = real3{vx, vy, vz};
        }
        __syncwarp();
    }
    // vertex distances to the centre, all at once
    #pragma unroll 1
    for (int vi = lane; vi < vn; vi += 32) {
        const real4 X = sh.vx[vi];
        sh.vx[vi].w = sqrt(X.x * X.x + X.y * X.y + X.z * X.z);
    }
    __syncwarp();

    // ---- arc points where edges leave the sphere (LIB/Vcontacts.cpp:418-462): the edges with an
    //      end outside the sphere listed in order, then their
    //      sphere intersections a warp at a time ----
    uint8_t* elist = sh.elist;
    int n_out = 0;
    #pragma unroll 1
    for (int e0 = 0; e0 < edgenum; e0 += 32) {
        const int e = e0 + lane;
        bool out = false;
        if (e < edgenum) {
            const uchar2 se = sh.u.e.es[e];
            out = rado < sh.vx[se.x].w || rado < sh.vx[se.y].w;
        }
        const unsigned m = __ballot_sync(kFull, out);
        if (out) elist[n_out + __popc(m & lanemask_lt())] = (uint8_t)e;
        n_out += __popc(m);
    }
    __syncwarp();
    #pragma unroll 1
    for (int k0 = 0; k0 < n_out; k0 += 32) {
        const int k = k0 + lane;
        int cnt = 0;
        real a0[3], a1[3];
        bool k0v = false, k1v = false;
        uchar4 q = make_uchar4(0, 0, 0, 0);
        if (k < n_out) {
            q = sh.u.e.ep[elist[k]];
            if (solve2s(sh.pl[q.x], sh.pl[q.y], rr, a0, a1)) {
                const real4 ta = sh.pl[q.z], tb = sh.pl[q.w];
                k0v = (dot3(ta, a0[0], a0[1], a0[2]) + ta.w < real(0.0)) && (dot3(tb, a0[0], a0[1], a0[2]) + tb.w < real(0.0));
                k1v = (dot3(ta, a1[0], a1[1], a1[2]) + ta.w < real(0.0)) && (dot3(tb, a1[0], a1[1], a1[2]) + tb.w < real(0.0));
                cnt = (int)k0v + (int)k1v;
            }
        }
        int tot;
        const int off = warp_excl_scan(cnt, lane, &tot);
        if (vn + tot > kMaxVerts - 1) return kAtomCapacity;
        int w = vn + off;
        if (k0v) {
            sh.vx[w] = make_real4(a0[0], a0[1], a0[2], rado);
            sh.vp[w] = make_uchar4(q.x, q.y, kNone, 0);
            ++w;
        }
        if (k1v) {
            sh.vx[w] = make_real4(a1[0], a1[1], a1[2], rado);
            sh.vp[w] = make_uchar4(q.x, q.y, kNone, 0);
        }
        vn += tot;
        __syncwarp();
    }
    // ---- keep the vertices inside the sphere, in order ----
    int nv = 0;
    #pragma unroll 1
    for (int v0 = 0; v0 < vn; v0 += 32) {
        const int vi = v0 + lane;
        real4 X = make_real4(0, 0, 0, 0);
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
    #pragma unroll 1
    for (int x0 = 0; x0 < NC; x0 += 32) {
        const int X = x0 + lane;
        int cnt = 0;
        if (X < NC && sh.flag[X] != 0)
            #pragma unroll 1
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
    // the faces' point lists and, for a face of more than two points, the antipode of its first
    // sphere point, which joins the face when it lies behind every other plane (test_point)
    int nf = 0;
    #pragma unroll 1
    for (int x0 = 0; x0 < NC; x0 += 32) {
        const int X = x0 + lane;
        bool cand = false;
        if (X < NC && sh.flag[X] != 0) {
            const int o = sh.foff[X];
            int k = 0;
            #pragma unroll 1
            for (int vi = 0; vi < NV; ++vi) {
                const uchar4 P = sh.vp[vi];
                if (P.x == X || P.y == X || P.z == X) sh.u.f.pt[o + k++] = (uint8_t)vi;
            }
            if (k > 2) {
                const real4 cp = centre_of(sh.pl[X]);
                #pragma unroll 1
                for (int q = 0; q < k; ++q) {
                    const int vi = sh.u.f.pt[o + q];
                    if (sh.vp[vi].z == kNone) {
                        const real4 pv = sh.vx[vi];
                        real* ex = &sh.u.f.cosv[3 * X];
                        ex[0] = real(2.0) * cp.x - pv.x;
                        ex[1] = real(2.0) * cp.y - pv.y;
                        ex[2] = real(2.0) * cp.z - pv.z;
                        cand = true;
                        break;
                    }
                }
            }
        }
        const unsigned m = __ballot_sync(kFull, cand);
        if (lane == 0) sh.cmask[x0 >> 5] = m;
        if (cand) sh.flist[nf + __popc(m & lanemask_lt())] = (uint8_t)X;
        nf += __popc(m);
    }
    __syncwarp();
    faces_inside(sh, NC, nf, lane);
    int n_extra = 0;
    #pragma unroll 1
    for (int x0 = 0; x0 < NC; x0 += 32) {
        const int X = x0 + lane;
        const bool extra = X < NC && ((sh.cmask[x0 >> 5] >> lane) & 1u) && !((sh.bad[x0 >> 5] >> lane) & 1u);
        int t;
        const int off = warp_excl_scan(extra ? 1 : 0, lane, &t);
        if (NV + n_extra + t > kMaxVerts - 1) return kAtomCapacity;
        if (extra) {
            const int w = NV + n_extra + off;
            if (hist) {
                hist_vx(hist)[w - NV] = sh.vx[w];
                hist_vp(hist)[w - NV] = sh.vp[w];
            }
            const real* ex = &sh.u.f.cosv[3 * X];
            sh.vx[w] = make_real4(ex[0], ex[1], ex[2], rado);
            sh.vp[w] = make_uchar4((uint8_t)X, kNone, kNone, 0);
            sh.u.f.pt[sh.foff[X] + sh.fnp[X]] = (uint8_t)w;
            sh.fnp[X] += 1;
        }
        n_extra += t;
    }
    __syncwarp();
    // ordering around each face (pt[0], a neighbour of it, then decreasing cosine): the second
    // point per face (one face per lane), the cosines of all faces' points spread over the lanes,
    // then each face's sort and its history (one face per lane)
    int np_miss = 0, np_lost = 0;
    #pragma unroll 1
    for (int X = lane; X < NC; X += 32) {
        if (sh.flag[X] == 0) continue;
        const int np = sh.fnp[X];
        uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
        int stale_prev = kNone;   // point 1 of the face before a replayed read of the slot past its end
        if (np > 3) {
            const uchar4 P0 = sh.vp[pt[0]];
            const int pY = (P0.x == X) ? P0.y : P0.x;
            int vi = 1;
            #pragma unroll 1
            for (; vi < np; ++vi) {
                const uchar4 q = sh.vp[pt[vi]];
                if (q.x == pY || q.y == pY || q.z == pY) break;
            }
            bool replayed = false;
            if (vi == np) {
                ++np_miss;
                const int s = (hist && np < kHistPts) ? (int)hist[X * kHistPts + np] : -1;
                if (s >= 0 && s < kMaxVerts - 1) {
                    // the reference swaps pt[1] with the stale slot: the slot's vertex becomes
                    // point 1, the old point 1 stays behind in the slot
                    replayed = true;
                    stale_prev = pt[1];
                    pt[1] = (uint8_t)s;
                } else {
                    if (hist) ++np_lost;
                    const int pZ = (P0.x == X || P0.y == X) ? P0.z : P0.y;
                    vi = 1;
                    if (pZ != kNone) {
                        int w = 1;
                        #pragma unroll 1
                        for (; w < np; ++w) {
                            const uchar4 q = sh.vp[pt[w]];
                            if (q.x == pZ || q.y == pZ || q.z == pZ) break;
                        }
                        if (w < np) vi = w;
                    }
                }
            }
            if (!replayed) {
                const uint8_t tmp = pt[vi];
                pt[vi] = pt[1];
                pt[1] = tmp;
            }
        }
        sh.sprev[X] = (uint8_t)stale_prev;
    }
    *no_partner += warp_sum(np_miss);
    *unreplayed += warp_sum(np_lost);
    __syncwarp();
    #pragma unroll 1
    for (int k0 = 0; k0 < tot_pts; k0 += 32) {
        const int k = k0 + lane;
        if (k < tot_pts) {
            const int X = face_of(sh.foff, NC, k);
            const int j = k - sh.foff[X];
            const int np = sh.fnp[X];
            if (sh.flag[X] != 0 && np > 3 && j >= 2 && j < np) {
                const uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
                // point 1 is read as it stood when the reference ordered this face: a replayed
                // slot that a later face's antipodal point takes still held its old vertex
                const int s1 = pt[1];
                const real4 v1 = (hist && s1 >= NV && s1 < NV + n_extra && sh.vp[s1].x > X) ? hist_vx(hist)[s1 - NV]
                                                                                          : sh.vx[s1];
                sh.u.f.cosv[sh.foff[X] + j] = cos_pqr(v1, sh.vx[pt[0]], sh.vx[pt[j]]);
            }
        }
    }
    __syncwarp();
    #pragma unroll 1
    for (int X = lane; X < NC; X += 32) {
        if (sh.flag[X] == 0) continue;
        const int np = sh.fnp[X];
        uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
        if (np > 3) {
            real* cs = &sh.u.f.cosv[sh.foff[X]];
            #pragma unroll 1
            for (int a = 2; a < np - 1; ++a)
                #pragma unroll 1
                for (int b = a + 1; b < np; ++b)
                    if (cs[a] < cs[b]) {
                        const uint8_t t = pt[a];
                        pt[a] = pt[b];
                        pt[b] = t;
                        const real tc = cs[a];
                        cs[a] = cs[b];
                        cs[b] = tc;
                    }
        }
        if (hist) {
            uint8_t* h = hist + X * kHistPts;
            const int nw = np < kHistPts ? np : kHistPts;
            #pragma unroll 1
            for (int k = 0; k < nw; ++k) h[k] = pt[k];
            if (sh.sprev[X] != kNone) h[np] = sh.sprev[X];
        }
    }
    __syncwarp();

    // ---- areas (LIB/Vcontacts.cpp:838-1044) ----
    // the first three engulfing planes in plane order
    int epi = 0;
    #pragma unroll 1
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
        real pp[3];
        if (epi == 1) {
            const real4 c = centre_of(sh.pl[sh.eng[0]]);
            pp[0] = c.x; pp[1] = c.y; pp[2] = c.z;
        } else if (epi == 2) {
            real q0[3], q1[3];
            if (!solve2s(sh.pl[sh.eng[0]], sh.pl[sh.eng[1]], rr, q0, q1)) {
                pp[0] = sh.vx[kMaxVerts - 1].x;   // atom-centre fallback, staged by the caller
                pp[1] = sh.vx[kMaxVerts - 1].y;
                pp[2] = sh.vx[kMaxVerts - 1].z;
            } else {
                pp[0] = (q0[0] + q1[0]) * real(0.5);   // the same value as / 2
                pp[1] = (q0[1] + q1[1]) * real(0.5);
                pp[2] = (q0[2] + q1[2]) * real(0.5);
            }
        } else {
            solve3(sh.pl[sh.eng[0]], sh.pl[sh.eng[1]], sh.pl[sh.eng[2]], pp);
        }
        #pragma unroll 1
        for (int vi = lane; vi < NV; vi += 32) {
            if (sh.vp[vi].z == kNone) continue;
            real4 P = sh.vx[vi];
            const real Vx = P.x - pp[0], Vy = P.y - pp[1], Vz = P.z - pp[2];
            const real a = Vx * Vx + Vy * Vy + Vz * Vz;
            const real b = 2 * (P.x * Vx + P.y * Vy + P.z * Vz);
            const real c = P.x * P.x + P.y * P.y + P.z * P.z - rr;
#if FXE_REFERENCE_FORMULAS
            const real k = (sqrt(b * b - real(4.0) * a * c) - b) / (2 * a);
#else
            // positive root of a k^2 + b k + c = 0 without cancellation when b > 0
            const real sq = sqrt(b * b - real(4.0) * a * c);
            const real k = b > real(0.0) ? (-real(2.0) * c) / (sq + b) : (sq - b) / (2 * a);
#endif
            P.x += k * Vx; P.y += k * Vy; P.z += k * Vz;
            P.w = rado;
            sh.vx[vi] = P;
        }
        __syncwarp();
    }
    const real two_pi_r = real(2.0) * (real)kPi * rado;
    // Caps and lenses (faces of 0 and 2 points) test their plane's centre against the other planes
    // (all faces' tests spread over the lanes); the fan triangles and arc segments of the other
    // faces, and the lenses' arcs, are laid out flat and spread over the lanes, then added to their
    // face's area in the reference's order (triangles, then arcs, each in point order).
    int t_run = 0, a_run = 0, nf2 = 0, n_lens = 0;
    #pragma unroll 1
    for (int x0 = 0; x0 < NC; x0 += 32) {
        const int X = x0 + lane;
        int nt = 0, na = 0;
        bool ring = false;
        if (X < NC && sh.flag[X] != 0) {
            const int np = sh.fnp[X];
            if (np == 0 || np == 2) {
                ring = true;
                const real4 cp = centre_of(sh.pl[X]);
                real* q = &sh.u.f.cosv[3 * X];
                q[0] = cp.x;
                q[1] = cp.y;
                q[2] = cp.z;
            } else {
                // (a face of one point has neither triangles nor arcs)
                const uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
                nt = np > 2 ? np - 2 : 0;
                #pragma unroll 1
                for (int vi = 0; vi < np; ++vi) na += arc_segment(sh, pt, np, vi);
            }
            sh.area[X] = real(0.0);
        }
        const unsigned m = __ballot_sync(kFull, ring);
        if (lane == 0) sh.cmask[x0 >> 5] = m;
        if (ring) sh.flist[nf2 + __popc(m & lanemask_lt())] = (uint8_t)X;
        nf2 += __popc(m);
        const bool lens = ring && sh.fnp[X] == 2;
        const unsigned ml = __ballot_sync(kFull, lens);
        if (lens) sh.llist[n_lens + __popc(ml & lanemask_lt())] = (uint8_t)X;
        n_lens += __popc(ml);
        int tt, ta;
        const int ot = warp_excl_scan(nt, lane, &tt);
        const int oa = warp_excl_scan(na, lane, &ta);
        if (X < NC) {
            sh.toff[X] = (uint16_t)(t_run + ot);
            sh.aoff[X] = (uint16_t)(a_run + oa);
        }
        t_run += tt;
        a_run += ta;
    }
    __syncwarp();
    faces_inside(sh, NC, nf2, lane);
    // caps: the whole cap when its centre is inside the polyhedron
    #pragma unroll 1
    for (int X = lane; X < NC; X += 32)
        if (((sh.cmask[X >> 5] >> (X & 31)) & 1u) && sh.fnp[X] == 0 && !((sh.bad[X >> 5] >> (X & 31)) & 1u))
            sh.area[X] = two_pi_r * (rado - fabs(sh.pl[X].w));
    __syncwarp();
    // fan of spherical triangles from pt[0] (LIB/Vcontacts.cpp:906-940)
    #pragma unroll 1
    for (int k0 = 0; k0 < t_run; k0 += 32) {
        const int k = k0 + lane;
        int X = -1;
        real v = real(0.0);
        if (k < t_run) {
            X = face_of(sh.toff, NC, k);
            const int vi = 1 + k - sh.toff[X];
            const uint8_t* pt = &sh.u.f.pt[sh.foff[X]];
            v = fan_triangle(sh.vx[pt[0]], sh.vx[pt[vi]], sh.vx[pt[vi + 1]], rado);
        }
        add_in_order(sh, X, v, lane);
    }
    // arc segments between consecutive arc points of different edges (:943-954), then the
    // lenses' arcs (the cap less the arc when the centre is inside, else the arc alone)
    #pragma unroll 1
    for (int k0 = 0; k0 < a_run + n_lens; k0 += 32) {
        const int k = k0 + lane;
        int F = -1, ia = 0, ib = 0;
        bool lens = false;
        if (k < a_run) {
            F = face_of(sh.aoff, NC, k);
            const int np = sh.fnp[F];
            const uint8_t* pt = &sh.u.f.pt[sh.foff[F]];
            int j = k - sh.aoff[F], vi = 0;
            #pragma unroll 1
            for (; vi < np - 1; ++vi)
                if (arc_segment(sh, pt, np, vi) && j-- == 0) break;
            ia = pt[vi];
            ib = pt[(vi + 1) % np];
        } else if (k < a_run + n_lens) {
            F = sh.llist[k - a_run];
            const uint8_t* pt = &sh.u.f.pt[sh.foff[F]];
            ia = pt[0];
            ib = pt[1];
            lens = true;
        }
        real v = real(0.0);
        if (F >= 0) v = sph_arc(centre_of(sh.pl[F]), sh.vx[ia], sh.vx[ib], rado);
        add_in_order(sh, lens ? -1 : F, v, lane);
        if (lens)
            sh.area[F] = ((sh.bad[F >> 5] >> (F & 31)) & 1u) ? v : two_pi_r * (rado - fabs(sh.pl[F].w)) - v;
    }
    __syncwarp();
    engulf_corrections(sh, NC, tot_pts, rado, rr, two_pi_r, epi, lane);
    sh.nv = NV;
    __syncwarp();
    return kAtomOk;
}

// Planes of the contacts of one scored atom (LIB/Vcontacts.cpp:186-221): the candidates whose
// bit in `excl` is clear (the list get_contlist4 gives; an excluded candidate is a saved atom that
// kept no contact with this one, or one at distance zero), packed in candidate order, so that
// each plane's index, and every tie-break on it, is the reference's contact index. Returns NC.
__device__ int load_planes(VorShared& sh, const DevSystem& S, const DevWork& W, int p, int a,
                           int n_cand, float4 me, float rado, const uint32_t* excl, int lane) {
    const int nm = n_mobile(S);
    const size_t cb = ((size_t)p * nm + a) * kMaxCand;
    const float rr = rado * rado;          // single-precision products, as in the reference
    int NC = 0;
    #pragma unroll 1
    for (int c0 = 0; c0 < n_cand; c0 += 32) {
        const int c = c0 + lane;
        const bool keep = c < n_cand && !((excl[c >> 5] >> (c & 31)) & 1u);
        const unsigned m = __ballot_sync(kFull, keep);
        if (keep) {
            const int r = NC + __popc(m & lanemask_lt());
            const int j = W.cand_idx[cb + c];
            const float d2 = W.cand_d2[cb + c];
            sh.cidx[r] = j;
            sh.cslot[r] = (uint8_t)c;
            const int mj = mobile_of(S, j);
            const float4 pj = mj < 0 ? S.rec_pos[j] : W.mob_pos[(size_t)p * nm + mj];
            const real d = sqrt((real)d2);
            const float q = kRw + pj.w;
            const float qq = q * q;
            // the reference squares the double distance; in single precision d2 itself is closer
            const real dd = sizeof(real) == 8 ? d * d : (real)d2;
            const real num = (dd + (real)rr) - (real)qq;
            bool eng = num < real(0.0);
            if (sizeof(real) < 8 && fabs(num) < real(1e-3)) eng = ((double)d2 + (double)rr) - (double)qq < 0.0;
            const real4 P = make_real4((real)(pj.x - me.x) / d, (real)(pj.y - me.y) / d, (real)(pj.z - me.z) / d,
                                       -(num / (real(2.0) * d)));
            sh.pl[r] = P;
#if FXE_FILTER
            sh.plf[r] = make_float4((float)P.x, (float)P.y, (float)P.z, (float)P.w);
#endif
            sh.flag[r] = eng ? kEngulf : 0;
        }
        NC += __popc(m);
    }
    // project_points' fallback centre for two engulfing planes: the atom's own coordinates + rado
    if (lane == 0) sh.vx[kMaxVerts - 1] = make_real4((real)(me.x + rado), (real)me.y, (real)me.z, real(0.0));
    __syncwarp();
    return NC;
}

__device__ double pose_clash_sum(const DevSystem& S, const DevWork& W, int p, int lane) {
    const int nm = n_mobile(S);
    double s = 0.0;
    #pragma unroll 1
    for (int m = lane; m < nm; m += 32) s += W.clash_part[(size_t)p * nm + m];
    return warp_sum(s);
}

// ------------------------------------------------------------------------------------------
// pose_kernel: calc_region + vcfunction for one pose per warp
// ------------------------------------------------------------------------------------------
// Shared memory per warp sets how many poses an SM holds at once, so the per-pose seeds and
// record masks live in the workspace (W.pose_seed, W.pose_rec); 20.0 KB of shared memory per pose
// in double precision, 11.1 KB in single.
struct PoseShared {
    VorShared v;
    uint8_t order[kMaxLig];          // mobile atoms in Calclist order
    uint32_t done[kMaskWords];       // mobile atoms whose contacts are saved
};

__device__ __forceinline__ bool bit(const uint32_t* m, int l) { return (m[l >> 5] >> (l & 31)) & 1u; }

__device__ __forceinline__ double get_yval(const DevSystem& S, int idx, double rel) {
    const int o = S.em_off[idx], e = S.em_off[idx + 1];
    if (S.em_weight[idx]) return (double)S.em_y[o];
    int k = o;
    while (k + 1 < e && rel > (double)S.em_x[k + 1]) ++k;
    if ((double)S.em_x[k] > rel) return 0.0;
    if (k + 1 >= e) return (double)S.em_y[k];
    return (double)S.em_y[k] + (rel - (double)S.em_x[k]) / (double)(S.em_x[k + 1] - S.em_x[k]) *
                                   (double)(S.em_y[k + 1] - S.em_y[k]);
}

__device__ void finish_failed(const DevWork& W, int p, int lane, int status, double wal) {
    fxe_cf cf;
    memset(&cf, 0, sizeof(cf));
    cf.status = status;
    if (status != FXE_POSE_CAPACITY) {
        // the reference's positional initialiser puts 1 into metal_coord (LIB/ic2cf.cpp:127-131)
        cf.wal = wal;
        cf.metal_coord = 1.0;
        cf.evalue = cf.wal + cf.metal_coord;
    }
    if (lane == 0) W.out[p] = cf;
}

// p < 0: no pose (the warp only keeps its block's barriers). n_iter: the atom steps the block
// takes together in lockstep (at least this pose's scored atoms; unused otherwise).
__device__ __forceinline__ void score_pose(const DevSystem& S, const DevWork& W, int p, int lane,
                                           PoseShared& ps, uint8_t* hist, int n_iter) {
    VorShared& sh = ps.v;
    // a pose that fails stops here; in lockstep its warp still meets the block after every step
    bool alive = p >= 0;
    if (p < 0) p = 0;
    const int nl = n_mobile(S);      // the scored atoms: side-chain atoms, then the ligand
    // polyhedron seeds (Calc indices, -1 = none) and the mobile partners each processed atom kept
    int (*const seed)[3] = reinterpret_cast<int (*)[3]>(W.pose_seed + (size_t)p * kMaxLig * 3);
    uint32_t (*const rec)[kMaskWords] = reinterpret_cast<uint32_t (*)[kMaskWords]>(W.pose_rec + (size_t)p * kMaxLig * kMaskWords);
    const size_t lb = (size_t)p * nl;
    if (alive && W.pose_grid[p].z) {
        finish_failed(W, p, lane, FXE_POSE_CAPACITY, 0.0);
        alive = false;
    }
    // clash pre-filter (LIB/Vcontacts.cpp:36-51)
    if (alive) {
        const double clash = pose_clash_sum(S, W, p, lane);
        if (clash >= kClashThreshold) {
            finish_failed(W, p, lane, FXE_POSE_CLASHED, clash);
            alive = false;
        }
    }
    if (!kLockstep && !alive) return;
    #pragma unroll 1
    for (int l = lane; alive && l < nl; l += 32) {
        ps.order[W.mob_rank[lb + l]] = (uint8_t)l;
        seed[l][0] = seed[l][1] = seed[l][2] = -1;
#pragma unroll
        for (int w = 0; w < kMaskWords; ++w) rec[l][w] = 0;
    }
    if (alive && lane < kMaskWords) ps.done[lane] = 0;
    // the face history starts the pose at zero, as the reference's ptorder does on a workspace
    // cleared before the pose
    if (alive && hist) {
        uint4* h4 = reinterpret_cast<uint4*>(hist);
        #pragma unroll 1
        for (int k = lane; k < kHistBytes / 16; k += 32) h4[k] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncwarp();
    // calc_region: atoms in Calclist order (LIB/Vcontacts.cpp:74-139)
    #pragma unroll 1
    for (int r = 0; r < (kLockstep ? n_iter : nl); ++r) {
        if (!alive || r >= nl) goto atom_end;
        {
        const int a = ps.order[r];
        const int n_cand = W.cand_n[lb + a];
        if (n_cand < 0) {
            if (lane == 0) atomicAdd(&W.counters[2], 1);
            finish_failed(W, p, lane, FXE_POSE_CAPACITY, 0.0);
            alive = false;
            goto atom_end;
        }
        const size_t cb = (lb + a) * kMaxCand;
        // get_contlist4's list: saved atoms drop out unless they kept a contact with this one, and
        // so does an atom at distance zero
        uint32_t excl[kMaxCand / 32];
        int kept_n = 0;
#pragma unroll
        for (int w = 0; w < kMaxCand / 32; ++w) {
            const int c = w * 32 + lane;
            bool ex = false;
            if (c < n_cand) {
                const int l = mobile_of(S, W.cand_idx[cb + c]);
                if (l >= 0) ex = bit(ps.done, l) && !bit(rec[l], a);
                if (W.cand_d2[cb + c] < 1e-20f) ex = true;
            }
            excl[w] = __ballot_sync(kFull, ex);
            kept_n += __popc(__ballot_sync(kFull, c < n_cand && !ex));
        }
        if (kept_n == 0) {   // no contacts: SAS -1, nothing saved, the atom is not marked done
            #pragma unroll 1
            for (int c = lane; c < n_cand; c += 32) {
                W.cand_area[cb + c] = 0.0;
                W.cand_flag[cb + c] = 0;
            }
            goto atom_end;
        }
        const float4 me = W.mob_pos[lb + a];
        const float rado = me.w + kRw;
        const int NC = load_planes(sh, S, W, p, a, n_cand, me, rado, excl, lane);
        // seed vertex left by an earlier atom, if all three of its planes are in the list
        int sA = -1, sB = -1, sC = -1;
        if (seed[a][0] != -1) {
            const int s0 = seed[a][0], s1 = seed[a][1], s2 = seed[a][2];
            #pragma unroll 1
            for (int c0 = 0; c0 < NC; c0 += 32) {
                const int c = c0 + lane;
                const int j = c < NC ? sh.cidx[c] : -2;
                const unsigned m0 = __ballot_sync(kFull, j == s0);
                const unsigned m1 = __ballot_sync(kFull, j == s1 && j != s0);
                const unsigned m2 = __ballot_sync(kFull, j == s2 && j != s0 && j != s1);
                if (m0) sA = c0 + 31 - __clz(m0);
                if (m1) sB = c0 + 31 - __clz(m1);
                if (m2) sC = c0 + 31 - __clz(m2);
            }
        }
        int np_miss = 0, np_lost = 0;
        const int st = voronoi_warp(sh, NC, rado, lane, &np_miss, &np_lost, sA, sB, sC, hist);
        if (lane == 0 && np_miss) atomicAdd(&W.counters[3], np_miss);
        if (lane == 0 && np_lost) atomicAdd(&W.counters[0], np_lost);
        if (st == kAtomCapacity) {
            if (lane == 0) atomicAdd(&W.counters[2], 1);
            finish_failed(W, p, lane, FXE_POSE_CAPACITY, 0.0);
            alive = false;
            goto atom_end;
        }
        if (st == kAtomHullFail) {
            if (lane == 0) atomicAdd(&W.counters[1], 1);
            finish_failed(W, p, lane, FXE_POSE_POLYHEDRON_FAILED, (double)kPolyPenalty);
            alive = false;
            goto atom_end;
        }
        // save_areas (LIB/Vcontacts.cpp:1149-1220): contacts with area > 0 on a contact plane;
        // candidates outside the contact list record nothing
        uint32_t keep_lig[kMaskWords] = {0, 0, 0, 0};
        #pragma unroll 1
        for (int c = lane; c < n_cand; c += 32) {
            if ((excl[c >> 5] >> (c & 31)) & 1u) {
                W.cand_area[cb + c] = 0.0;
                W.cand_flag[cb + c] = 0;
            }
        }
        #pragma unroll 1
        for (int k = lane; k < NC; k += 32) {
            const real ar = sh.area[k];
            const uint8_t f = sh.flag[k];
            const bool kept = ar > real(0.0) && (f & (kOnHull | kEngulf));
            const int c = sh.cslot[k];
            W.cand_area[cb + c] = (double)ar;
            W.cand_flag[cb + c] = (uint8_t)(f | (kept ? kRecorded : 0));
            const int l = kept ? mobile_of(S, sh.cidx[k]) : -1;
            if (l >= 0) keep_lig[l >> 5] |= 1u << (l & 31);
        }
#pragma unroll
        for (int w = 0; w < kMaskWords; ++w) {
            uint32_t m = keep_lig[w];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m |= __shfl_xor_sync(kFull, m, o);
            if (lane == 0) rec[a][w] = m;
        }
        // save_seeds (LIB/Vcontacts.cpp:601-629): first vertex naming each later atom's plane
        if (lane == 0) {
            const int az = slot_of(S, a);
            #pragma unroll 1
            for (int vi = 0; vi < sh.nv; ++vi) {
                const uchar4 q = sh.vp[vi];
                if (q.z == kNone || q.x >= NC || q.y >= NC || q.z >= NC) continue;
                const int j0 = sh.cidx[q.x], j1 = sh.cidx[q.y], j2 = sh.cidx[q.z];
                const int m0 = mobile_of(S, j0), m1 = mobile_of(S, j1), m2 = mobile_of(S, j2);
                if (m0 >= 0 && seed[m0][0] == -1) {
                    seed[m0][0] = az; seed[m0][1] = j1; seed[m0][2] = j2;
                }
                if (m1 >= 0 && seed[m1][0] == -1) {
                    seed[m1][0] = az; seed[m1][1] = j0; seed[m1][2] = j2;
                }
                if (m2 >= 0 && seed[m2][0] == -1) {
                    seed[m2][0] = az; seed[m2][1] = j0; seed[m2][2] = j1;
                }
            }
            ps.done[a >> 5] |= 1u << (a & 31);
        }
        __syncwarp();
    }
    atom_end:
        if (kLockstep) __syncthreads();
        if (!kLockstep && !alive) return;
    }
    if (!alive) return;
    // vcfunction (LIB/vcfunction.cpp:84-513): scored atoms in Calc order (side-chain atoms,
    // then the ligand), their kept contacts; each residue's terms are summed on their own and the
    // records added up ligand first, then the side chains in order (LIB/ic2cf.cpp:133-245)
    const int T = S.ntypes, nsc = S.n_sc;
    const double permea = (double)S.permeability;
    double com = 0.0, wal = 0.0, sas = 0.0, totsas = 0.0;
    double res_com[kMaxFlex], res_wal[kMaxFlex], res_sas[kMaxFlex];
#pragma unroll
    for (int r = 0; r < kMaxFlex; ++r) res_com[r] = res_wal[r] = res_sas[r] = 0.0;
    int cur_res = -1;
    #pragma unroll 1
    for (int i = 0; i < nl; ++i) {
        const int NC = W.cand_n[lb + i];
        const size_t cb = (lb + i) * kMaxCand;
        const bool side = i < nsc;
        const int res = side ? S.sc_res[i] : kMaxFlex;
        if (res != cur_res) {
            if (cur_res >= 0 && cur_res < kMaxFlex) {
                res_com[cur_res] = com;
                res_wal[cur_res] = wal;
                res_sas[cur_res] = sas;
            }
            com = wal = sas = 0.0;
            cur_res = res;
        }
        const double radA = (double)W.mob_pos[lb + i].w;
        const double radoA = radA + (double)kRw;
        const double surfA = 4.0 * kPi * radoA * radoA;
        const int ti = side ? S.rec_type[S.sc_slot[i]] : S.lig_type[i - nsc];
        double c_com = 0.0, c_wal = 0.0, c_area = 0.0;
        #pragma unroll 1
        for (int c = lane; c < NC; c += 32) {
            if (!(W.cand_flag[cb + c] & kRecorded)) continue;
            const int j = W.cand_idx[cb + c];
            const double area = (double)W.cand_area[cb + c];
            c_area += area;
            const int rel = residue_pair(S, i, j);
            if (rel == 1) continue;                      // bonded within the residue
            const int mj = mobile_of(S, j);
            if (mj >= 0 && mj < i) continue;             // FA->contacts: scored from that atom
            const bool lig_j = j >= S.n_rec;
            const float rj = lig_j ? S.lig_radius[j - S.n_rec] : (mj >= 0 ? W.mob_pos[lb + mj].w : S.rec_pos[j].w);
            const int tj = lig_j ? S.lig_type[j - S.n_rec] : S.rec_type[j];
            const int eidx = (ti - 1) * T + (tj - 1);
            // intramolecular: one residue, or two protein residues (LIB/vcfunction.cpp:283-291)
            const bool intra = rel != 0 || (side && !lig_j);
            if (S.intramolecular || !intra) {
                const double yval = get_yval(S, eidx, area / surfA);
                c_com += S.em_weight[eidx] ? yval * area : yval;
            }
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
        if (!side) totsas += SAS;
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
    // the ligand's record (com/wal/sas hold it now), then each side chain's
    #pragma unroll 1
    for (int r = 0; r < S.n_flex; ++r) {
        com += res_com[r];
        wal += res_wal[r];
        sas += res_sas[r];
    }
    fxe_cf cf;
    memset(&cf, 0, sizeof(cf));
    cf.com = com;
    cf.wal = wal;
    cf.sas = sas;
    cf.totsas = totsas;
    cf.evalue = cf.com + cf.wal + cf.sas + cf.con + cf.elec + cf.hbond + cf.gist_desolv + cf.metal_coord;
    cf.status = FXE_POSE_SCORED;
    if (lane == 0) W.out[p] = cf;
}

// Poses are handed out from a queue (`next`, zeroed before the launch): the launch keeps only as
// many blocks as the SMs hold at once, and each warp takes the next pose when it finishes one.
// Pose times vary several-fold, so this fills the SMs to the end of the launch where a grid of
// one block per pose pair left a partial last wave and idle SMs behind the slowest poses.
__device__ __forceinline__ int next_pose(int* next, int lane) {
    int p = 0;
    if (lane == 0) p = atomicAdd(next, 1);
    return __shfl_sync(kFull, p, 0);
}

// The warp's face history (hist_all: kHistStride bytes per warp of the launch), or null.
__device__ __forceinline__ uint8_t* warp_hist(uint8_t* hist_all) {
    return hist_all ? hist_all + (size_t)(blockIdx.x * kVorWarps + (threadIdx.x >> 5)) * kHistStride : nullptr;
}

// tile: poses a lockstep block takes at a time (its first `tile` warps score them; the others
// keep meeting the barriers); unused without lockstep.
__global__ void __launch_bounds__(kVorWarps * 32)
pose_kernel(DevSystem S, DevWork W, int n, int* next, uint8_t* hist_all, int tile) {
    extern __shared__ __align__(16) unsigned char smem[];
    PoseShared& ps = reinterpret_cast<PoseShared*>(smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    uint8_t* hist = warp_hist(hist_all);
    if (kLockstep) {
        // the block takes `tile` neighbouring poses of the queue at once
        __shared__ int base_s;
        #pragma unroll 1
        for (;;) {
            if (threadIdx.x == 0) base_s = atomicAdd(next, tile);
            __syncthreads();
            const int base = base_s;
            __syncthreads();
            if (base >= n) break;
            const int w = (int)(threadIdx.x >> 5);
            const int q = w < tile ? base + w : n;
            score_pose(S, W, q < n ? W.pose_order[q] : -1, lane, ps, hist, n_mobile(S));
            __syncwarp();
        }
    } else {
        #pragma unroll 1
        for (int q = next_pose(next, lane); q < n; q = next_pose(next, lane)) {
            score_pose(S, W, W.pose_order[q], lane, ps, hist, 0);
            __syncwarp();
        }
    }
}

// The same over the poses of several jobs; the job's system and workspace descriptors are read
// from the job table (they stay in L1), keeping shared memory for the polyhedron workspace.
__global__ void __launch_bounds__(kVorWarps * 32)
pose_kernel_jobs(const Job* __restrict__ jobs, int n_jobs, int total, int* next, const int* __restrict__ order,
                 uint8_t* hist_all, int tile) {
    extern __shared__ __align__(16) unsigned char smem[];
    PoseShared& ps = reinterpret_cast<PoseShared*>(smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    uint8_t* hist = warp_hist(hist_all);
    if (kLockstep) {
        // the block takes `tile` neighbouring poses of the queue at once and steps through as
        // many atoms as the largest of them has
        __shared__ int base_s, steps_s;
        #pragma unroll 1
        for (;;) {
            if (threadIdx.x == 0) {
                base_s = atomicAdd(next, tile);
                steps_s = 0;
            }
            __syncthreads();
            const int base = base_s;
            const int w = (int)(threadIdx.x >> 5);
            const int q = w < tile ? base + w : total;
            int gp = -1, j = 0;
            if (q < total) {
                gp = order[q];
                j = find_job(jobs, n_jobs, gp, false);
                if (lane == 0) atomicMax(&steps_s, n_mobile(jobs[j].S));
            }
            __syncthreads();
            const int steps = steps_s;
            __syncthreads();
            if (base >= total) break;
            const Job& job = jobs[j];
            score_pose(job.S, job.W, gp < 0 ? -1 : gp - job.pose0, lane, ps, hist, steps);
            __syncwarp();
        }
    } else {
        #pragma unroll 1
        for (int q = next_pose(next, lane); q < total; q = next_pose(next, lane)) {
            const int gp = order[q];
            const Job& job = jobs[find_job(jobs, n_jobs, gp, false)];
            score_pose(job.S, job.W, gp - job.pose0, lane, ps, hist, 0);
            __syncwarp();
        }
    }
}

size_t pose_smem_bytes() { return sizeof(PoseShared) * kVorWarps; }
size_t pose_jobs_smem_bytes() { return sizeof(PoseShared) * kVorWarps; }

static int g_resident_blocks = 0;   // blocks of pose_kernel the device holds at once
static int g_sms = 0, g_per_sm = 0;  // SMs, and blocks of pose_kernel one SM holds

// Blocks of a launch over n poses: no more than the device holds at once (the warps take poses
// from a queue), no more than blocks_per_sm per SM when that is set (> 0; the autotuner's
// occupancy cap), and no more than the face history holds (hist_bytes; 0: no history).
// Blocks a launch may run at once: as many as the device holds, no more than blocks_per_sm per
// SM when that is set (> 0), no more than the face history holds (hist_bytes; 0: no history).
static int pose_max_blocks(size_t hist_bytes, int blocks_per_sm) {
    int b = g_resident_blocks > 0 ? g_resident_blocks : 1;
    if (blocks_per_sm > 0 && g_sms > 0 && blocks_per_sm < g_per_sm && g_sms * blocks_per_sm < b)
        b = g_sms * blocks_per_sm;
    if (hist_bytes) {
        const size_t cap = hist_bytes / (kVorWarps * kHistStride);
        if ((size_t)b > cap) b = (int)cap;
    }
    return b > 0 ? b : 1;
}

// Poses a lockstep block takes at a time (0 without lockstep): all its warps' worth, or fewer
// when the launch's poses would not reach every block the device runs at once, so that they
// spread over more SMs (a pose's time is its chain of atoms, shorter with fewer warps sharing the
// SM's double-precision pipe).
int pose_tile_for(int n, size_t hist_bytes, int blocks_per_sm) {
    if (!kLockstep) return 0;
    if (hist_bytes < kVorWarps * kHistStride) hist_bytes = 0;
    const int r = pose_max_blocks(hist_bytes, blocks_per_sm);
    const int t = (int)(((long long)n + r - 1) / r);
    return t < 1 ? 1 : (t > kVorWarps ? kVorWarps : t);
}

// Blocks of a launch over n poses: one per tile of poses (per kVorWarps poses without lockstep),
// no more than pose_max_blocks.
static unsigned pose_blocks(int n, size_t hist_bytes, int blocks_per_sm) {
    const int per = kLockstep ? pose_tile_for(n, hist_bytes, blocks_per_sm) : kVorWarps;
    int b = (n + per - 1) / per;
    const int r = pose_max_blocks(hist_bytes, blocks_per_sm);
    if (b > r) b = r;
    return (unsigned)(b > 0 ? b : 1);
}

size_t pose_hist_bytes() { return (size_t)g_resident_blocks * kVorWarps * kHistStride; }
// The blocks of a launch.
int pose_launch_blocks(int n, size_t hist_bytes, int blocks_per_sm) {
    if (hist_bytes < kVorWarps * kHistStride) hist_bytes = 0;
    return (int)pose_blocks(n, hist_bytes, blocks_per_sm);
}
int pose_max_blocks_per_sm() { return g_per_sm; }
int pose_warps_per_block() { return kVorWarps; }

// hist / hist_bytes: the launch's face history (reference face order), or null / 0;
// blocks_per_sm: occupancy cap (0: as many as fit).
void launch_poses(const DevSystem& S, const DevWork& W, int n, int* next, uint8_t* hist, size_t hist_bytes,
                  int blocks_per_sm, cudaStream_t st) {
    if (hist_bytes < kVorWarps * kHistStride) hist = nullptr;
    if (!hist) hist_bytes = 0;
    cudaMemsetAsync(next, 0, sizeof(int), st);
    pose_kernel<<<pose_blocks(n, hist_bytes, blocks_per_sm), kVorWarps * 32, pose_smem_bytes(), st>>>(
        S, W, n, next, hist, pose_tile_for(n, hist_bytes, blocks_per_sm));
}

void launch_poses_jobs(const Job* jobs, int n_jobs, int total, int* next, const int* order, uint8_t* hist,
                       size_t hist_bytes, int blocks_per_sm, cudaStream_t st) {
    if (hist_bytes < kVorWarps * kHistStride) hist = nullptr;
    if (!hist) hist_bytes = 0;
    cudaMemsetAsync(next, 0, sizeof(int), st);
    pose_kernel_jobs<<<pose_blocks(total, hist_bytes, blocks_per_sm), kVorWarps * 32, pose_jobs_smem_bytes(), st>>>(
        jobs, n_jobs, total, next, order, hist, pose_tile_for(total, hist_bytes, blocks_per_sm));
}

cudaError_t configure_voronoi() {
    cudaError_t e = cudaFuncSetAttribute(pose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pose_smem_bytes());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(pose_kernel_jobs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pose_jobs_smem_bytes());
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pose_kernel, kVorWarps * 32, pose_smem_bytes())) != cudaSuccess)
        return e;
    g_sms = sms;
    g_per_sm = per_sm > 0 ? per_sm : 1;
    g_resident_blocks = sms * g_per_sm;
    return cudaSuccess;
}

}  // namespace FXE_VARIANT
}  // namespace fxe
