/* fxe_oracle.c — CPU restatement of the FlexAID∆S fitness-evaluation path (the checker).
 *
 * TEST INFRASTRUCTURE ONLY (see fxe_oracle.h). Each function restates the reference function
 * named in its comment, keeping the reference's order of operations and its float/double
 * types expression by expression, because parity with the reference is pinned to the bit on
 * ordinary inputs. Built with -ffp-contract=off so the compiler does not fuse operations.
 *
 * The reference runs one pose at a time through:
 *   ic2cf (LIB/ic2cf.cpp:18-386) -> buildcc (LIB/buildcc.cpp:6-134) -> vcfunction
 *   (LIB/vcfunction.cpp:14-574) -> Vcontacts (LIB/Vcontacts.cpp:6-64) with index_protein,
 *   get_contlist4, voronoi_poly2, order_faces, calc_areas, save_areas.
 * This file keeps that sequential structure, including the order-dependent 'done' marking and
 * polyhedron seeds, so that it reproduces the reference's contact lists and scores exactly.
 */
#include "fxe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define O_RW 1.4f                 /* LIB/flexaid.h:88 */
#define O_PI 3.141592             /* LIB/flexaid.h:86 */
#define O_KWALL 1.0e6f            /* LIB/flexaid.h:78 */
#define O_CELL 6.5f               /* LIB/Vcontacts.h:56 */
#define O_CLASH_THRESHOLD 1e4     /* LIB/flexaid.h:70 */
#define O_POLY_PENALTY 1e6f       /* LIB/flexaid.h:69 */
#define O_MAX_POLY 2200           /* LIB/Vcontacts.h:54 */
#define O_MAX_CONT 100            /* LIB/Vcontacts.h:52 */
#define O_MAX_EDGES 200           /* LIB/Vcontacts.cpp:378 */
#define O_MAX_FLEX 8              /* flexible side chains the descriptor may carry */

static int g_compat = 0;

void fxo_set_reference_compat(int on) { g_compat = on; }

/* Trigonometry of the pose build. The reference calls the C library's cosf/sinf
   (LIB/buildcc.cpp:80-100), whose last bit is not correctly rounded for about 1% of
   arguments and differs between C libraries. Mode 1 uses the correctly rounded values
   (double-precision cos/sin rounded once to float), the values the CUDA build kernel uses. */
static int g_trig_cr = 0;

void fxo_set_trig_rounding(int correctly_rounded) { g_trig_cr = correctly_rounded; }

static float o_cosf(float x) { return g_trig_cr ? (float)cos((double)x) : cosf(x); }
static float o_sinf(float x) { return g_trig_cr ? (float)sin((double)x) : sinf(x); }

typedef struct { double Ai[4]; double dist; int index; double area; char flag; } Plane;
typedef struct { double xi[3]; double dist; int plane[3]; } Vert;
typedef struct { double V[3]; int startpt, endpt, plane[2], startplane, endplane; char arc; } Edge;
typedef struct { int prev, atom, from; double area, dist; } CaRec;
typedef struct { int index; double dist; } Cand;
typedef struct { int numpts; int pt[O_MAX_CONT]; } PtOrder;

typedef struct {
    int natoms, nrec, nlig;
    /* per Calc slot: scored (ligand and side-chain atoms), residue (-1 a rigid one-atom residue,
       r a flexible side chain, n_flex the ligand), index in the residue, scored-atom index */
    char* score;
    int* res_of;
    int* loc;
    int* mob;
    int nflex;
    const fxe_flex_residue* flex;
    float (*xyz)[3];
    const float* radius;      /* Calc-order radii (receptor then ligand) */
    const int* type;
    float* rad_all;
    int* type_all;
    char* done;
    int* boxnum;
    int* calclist;
    int* ca_index;
    int* seed;
    CaRec* carec;
    int ncarec, carec_cap;
    Cand* cand;
    Plane* cont;
    Vert* poly;
    Edge* vedge;
    Vert* centerpt;
    PtOrder* ptorder;
    int* box_n;
    int* box_f;
    int box_cap;
    int dim;
    float (*lic)[3];          /* ligand dis, ang, dih */
    fxo_counts* counts;
} State;

/* ----------------------------------------------------------------------------------------
 * small geometry helpers (LIB/Vcontacts.cpp)
 * -------------------------------------------------------------------------------------- */

/* solve_3x3, LIB/Vcontacts.cpp:1384-1414: intersection of three planes (Cramer's rule). */
int fxo_solve_3x3(const double* e0, const double* e1, const double* e2, double* pt) {
    double c00 = e1[1] * e2[2] - e2[1] * e1[2];
    double c01 = -e1[0] * e2[2] + e2[0] * e1[2];
    double c02 = e1[0] * e2[1] - e2[0] * e1[1];
    double c10 = -e0[1] * e2[2] + e2[1] * e0[2];
    double c11 = e0[0] * e2[2] - e2[0] * e0[2];
    double c12 = -e0[0] * e2[1] + e2[0] * e0[1];
    double c20 = e0[1] * e1[2] - e1[1] * e0[2];
    double c21 = -e0[0] * e1[2] + e1[0] * e0[2];
    double c22 = e0[0] * e1[1] - e1[0] * e0[1];
    double det = e0[0] * c00 + e0[1] * c01 + e0[2] * c02;
    if (det == 0.0) return -1;
    pt[0] = -(e0[3] * c00 + e1[3] * c10 + e2[3] * c20) / det;
    pt[1] = -(e0[3] * c01 + e1[3] * c11 + e2[3] * c21) / det;
    pt[2] = -(e0[3] * c02 + e1[3] * c12 + e2[3] * c22) / det;
    return 0;
}

/* solve_2xS, LIB/Vcontacts.cpp:1427-1476: the two points where the line of two planes meets
 * the sphere of radius rado about the origin. */
int fxo_solve_2xS(const double* a, const double* b, float rado, double* pt0, double* pt1) {
    double e2[3];
    e2[0] = a[1] * b[2] - a[2] * b[1];
    e2[1] = a[2] * b[0] - a[0] * b[2];
    e2[2] = a[0] * b[1] - a[1] * b[0];
    double c00 = b[1] * e2[2] - e2[1] * b[2];
    double c01 = -b[0] * e2[2] + e2[0] * b[2];
    double c02 = b[0] * e2[1] - e2[0] * b[1];
    double c10 = -a[1] * e2[2] + e2[1] * a[2];
    double c11 = a[0] * e2[2] - e2[0] * a[2];
    double c12 = -a[0] * e2[1] + e2[0] * a[1];
    double det = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
    if (det == 0.0) return -1;
    double avg[3];
    avg[0] = -(a[3] * c00 + b[3] * c10) / det;
    avg[1] = -(a[3] * c01 + b[3] * c11) / det;
    avg[2] = -(a[3] * c02 + b[3] * c12) / det;
    double t = (rado * rado - avg[0] * avg[0] - avg[1] * avg[1] - avg[2] * avg[2]) / det;
    if (t < 0.0) return -1;
    t = sqrt(t);
    for (int k = 0; k < 3; ++k) {
        pt0[k] = avg[k] + t * e2[k];
        pt1[k] = avg[k] - t * e2[k];
    }
    return 0;
}

/* cosPQR, LIB/Vcontacts.cpp:1486-1505: cosine of the angle P-Q-R at Q. */
double fxo_cosPQR(const double* p, const double* q, const double* r) {
    double qp[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
    double qr[3] = {r[0] - q[0], r[1] - q[1], r[2] - q[2]};
    return (qp[0] * qr[0] + qp[1] * qr[1] + qp[2] * qr[2]) /
           sqrt((qp[0] * qp[0] + qp[1] * qp[1] + qp[2] * qp[2]) *
                (qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2]));
}

/* spherical_arc, LIB/Vcontacts.cpp:1518-1557: area between the great-circle arc B-C and the
 * small-circle arc of the cap centred on Ao. */
static double sph_arc(const Vert* ao, const Vert* b, const Vert* c, float rado) {
    double cosAOB = (ao->xi[0] * b->xi[0] + ao->xi[1] * b->xi[1] + ao->xi[2] * b->xi[2]) / (ao->dist * b->dist);
    double cosBOC = (b->xi[0] * c->xi[0] + b->xi[1] * c->xi[1] + b->xi[2] * c->xi[2]) / (b->dist * c->dist);
    double U = (1 + cosAOB) * sqrt((1 + cosBOC) / 8.0);
    double V = (1 - cosAOB) * sqrt((1 + cosBOC) / 8.0);
    double W = sqrt((1 - cosAOB) * (1 + cosAOB) * (1 - cosBOC) / 8.0);
    double tS = (1 - U + V + W + W) / (1 + U - V - W - W);
    double tSB = (1 - U - V) / (1 + U + V);
    double tSA = (1 - U + V - W - W) / (1 + U - V + W + W);
    double tanprod;
    if ((tS * tSA) > 0.0) tanprod = sqrt(tSB * tSB * tS * tSA);
    else tanprod = 0.0f;
    double cosBAC = fxo_cosPQR(b->xi, ao->xi, c->xi);
    double angBAC;
    if (cosBAC > 1.0) angBAC = 0.0f;
    else if (cosBAC < -1.0) angBAC = O_PI;
    else angBAC = acos(cosBAC);
    return rado * (angBAC * (rado - ao->dist) - 4.0 * rado * atan(sqrt(tanprod)));
}

double fxo_spherical_arc(const double* ao, double ao_dist, const double* b, double b_dist,
                         const double* c, double c_dist, float rado) {
    Vert A = {{ao[0], ao[1], ao[2]}, ao_dist, {0, 0, 0}};
    Vert B = {{b[0], b[1], b[2]}, b_dist, {0, 0, 0}};
    Vert Cc = {{c[0], c[1], c[2]}, c_dist, {0, 0, 0}};
    return sph_arc(&A, &B, &Cc, rado);
}

/* add_vertex, LIB/Vcontacts.cpp:680-690 */
static void add_vertex(Vert* poly, int vn, const double* x, int a, int b, int c) {
    poly[vn].xi[0] = x[0];
    poly[vn].xi[1] = x[1];
    poly[vn].xi[2] = x[2];
    poly[vn].plane[0] = a;
    poly[vn].plane[1] = b;
    poly[vn].plane[2] = c;
    poly[vn].dist = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
}

/* add_vedge, LIB/Vcontacts.cpp:642-672: new edge along the line of planes p0, p1, oriented
 * away from testplane. */
static void add_vedge(Edge* e, int en, const Plane* cont, int p0, int p1, int tp,
                      const Vert* poly, int sp) {
    e[en].V[0] = cont[p0].Ai[1] * cont[p1].Ai[2] - cont[p0].Ai[2] * cont[p1].Ai[1];
    e[en].V[1] = cont[p0].Ai[2] * cont[p1].Ai[0] - cont[p0].Ai[0] * cont[p1].Ai[2];
    e[en].V[2] = cont[p0].Ai[0] * cont[p1].Ai[1] - cont[p0].Ai[1] * cont[p1].Ai[0];
    e[en].startpt = sp;
    e[en].endpt = -1;
    e[en].plane[0] = p0;
    e[en].plane[1] = p1;
    e[en].startplane = tp;
    e[en].arc = '.';
    double t[3] = {poly[sp].xi[0] + e[en].V[0], poly[sp].xi[1] + e[en].V[1], poly[sp].xi[2] + e[en].V[2]};
    double tv = cont[tp].Ai[0] * t[0] + cont[tp].Ai[1] * t[1] + cont[tp].Ai[2] * t[2] + cont[tp].Ai[3];
    if (tv > 0.0) {
        e[en].V[0] = -e[en].V[0];
        e[en].V[1] = -e[en].V[1];
        e[en].V[2] = -e[en].V[2];
    }
}

/* test_point, LIB/Vcontacts.cpp:1357-1372: 'Y' unless the point lies behind a contact plane. */
static char test_point(const double* x, const Plane* cont, int NC, int pa, int pb, int pc) {
    for (int cp = 0; cp < NC; ++cp) {
        if (cp != pa && cp != pb && cp != pc && cont[cp].flag != 'X') {
            if ((cont[cp].Ai[0] * x[0] + cont[cp].Ai[1] * x[1] + cont[cp].Ai[2] * x[2] + cont[cp].Ai[3]) > 0.0)
                return 'N';
        }
    }
    return 'Y';
}

/* ----------------------------------------------------------------------------------------
 * Vcontacts
 * -------------------------------------------------------------------------------------- */

/* get_firstvert, LIB/Vcontacts.cpp:498-592: starting vertex from a seed, else from the plane
 * closest to the origin, the nearest edge on it and the nearest third plane along that edge. */
static void get_firstvert(const int* seed, const Plane* cont, int* pA, int* pB, int* pC, int NC,
                          int az) {
    int si = az * 3;
    *pA = -1;
    *pB = -1;
    *pC = -1;
    if (seed[si] != -1) {
        for (int c = 0; c < NC; ++c) {
            if (cont[c].index == seed[si]) *pA = c;
            else if (cont[c].index == seed[si + 1]) *pB = c;
            else if (cont[c].index == seed[si + 2]) *pC = c;
        }
    }
    if (*pA != -1 && *pB != -1 && *pC != -1) return;
    double mindist = 9.9e+9;
    for (int c = 0; c < NC; ++c)
        if (cont[c].dist < mindist) {
            mindist = cont[c].dist;
            *pA = c;
        }
    double ptA[3] = {0.0, 0.0, 0.0}, v[4], tmp[3];
    mindist = 9.9e+9;
    for (int c = 0; c < NC + 4; ++c) {
        if (c == *pA) continue;
        v[0] = cont[*pA].Ai[1] * cont[c].Ai[2] - cont[*pA].Ai[2] * cont[c].Ai[1];
        v[1] = cont[*pA].Ai[2] * cont[c].Ai[0] - cont[*pA].Ai[0] * cont[c].Ai[2];
        v[2] = cont[*pA].Ai[0] * cont[c].Ai[1] - cont[*pA].Ai[1] * cont[c].Ai[0];
        v[3] = 0.0;
        if (fxo_solve_3x3(cont[*pA].Ai, cont[c].Ai, v, tmp) != -1) {
            double d = sqrt(tmp[0] * tmp[0] + tmp[1] * tmp[1] + tmp[2] * tmp[2]);
            if (d < mindist) {
                *pB = c;
                mindist = d;
                ptA[0] = tmp[0];
                ptA[1] = tmp[1];
                ptA[2] = tmp[2];
            }
        }
    }
    v[0] = cont[*pA].Ai[1] * cont[*pB].Ai[2] - cont[*pA].Ai[2] * cont[*pB].Ai[1];
    v[1] = cont[*pA].Ai[2] * cont[*pB].Ai[0] - cont[*pA].Ai[0] * cont[*pB].Ai[2];
    v[2] = cont[*pA].Ai[0] * cont[*pB].Ai[1] - cont[*pA].Ai[1] * cont[*pB].Ai[0];
    v[3] = 0.0;
    double vtmin = 9.9e+9;
    for (int c = 0; c < NC + 4; ++c) {
        if (c != *pA && c != *pB) {
            double den = cont[c].Ai[0] * v[0] + cont[c].Ai[1] * v[1] + cont[c].Ai[2] * v[2];
            if (den != 0.0) {
                double vt = -(cont[c].Ai[0] * ptA[0] + cont[c].Ai[1] * ptA[1] + cont[c].Ai[2] * ptA[2] + cont[c].Ai[3]) / den;
                if (fabs(vt) < vtmin) {
                    vtmin = fabs(vt);
                    *pC = c;
                }
            }
        }
    }
}

/* save_seeds, LIB/Vcontacts.cpp:601-629 */
static void save_seeds(int* seed, const Plane* cont, const Vert* poly, int NV, int az) {
    for (int vi = 0; vi < NV; ++vi) {
        if (poly[vi].plane[2] == -1) continue;
        const int p0 = poly[vi].plane[0], p1 = poly[vi].plane[1], p2 = poly[vi].plane[2];
        int si = 3 * cont[p0].index;
        if (seed[si] == -1) { seed[si] = az; seed[si + 1] = cont[p1].index; seed[si + 2] = cont[p2].index; }
        si = 3 * cont[p1].index;
        if (seed[si] == -1) { seed[si] = az; seed[si + 1] = cont[p0].index; seed[si + 2] = cont[p2].index; }
        si = 3 * cont[p2].index;
        if (seed[si] == -1) { seed[si] = az; seed[si + 1] = cont[p0].index; seed[si + 2] = cont[p1].index; }
    }
}

/* voronoi_poly2, LIB/Vcontacts.cpp:147-490 (extended radical planes, planedef 'X'). Returns
 * the vertex count, or -1 when the hull walk reaches 200 edges (no recalculation after the
 * first call, LIB/top.cpp:1133). */
static int voronoi_poly2(State* S, int az, float rado, int NC) {
    Plane* cont = S->cont;
    Vert* poly = S->poly;
    Edge* ve = S->vedge;
    const Cand* cl = S->cand;
    int pA = -1, pB = -1, pC = -1, oldC;
    double mindist = 9.9e+9;
    for (int c = 0; c < NC; ++c) {
        const int j = cl[c].index;
        const double ad = cl[c].dist;
        if (ad < 1.0e-10) continue;
        const float rj = S->rad_all[j];
        double pd = (ad * ad + rado * rado - (O_RW + rj) * (O_RW + rj)) / (2 * ad);
        cont[c].Ai[0] = (S->xyz[j][0] - S->xyz[az][0]) / ad;
        cont[c].Ai[1] = (S->xyz[j][1] - S->xyz[az][1]) / ad;
        cont[c].Ai[2] = (S->xyz[j][2] - S->xyz[az][2]) / ad;
        cont[c].Ai[3] = -pd;
        cont[c].dist = fabs(pd);
        cont[c].index = j;
        cont[c].flag = 'X';
        if (cont[c].dist < mindist) {
            mindist = cont[c].dist;
            pA = c;
        }
    }
    static const double bound[4][4] = {{0.707, 1.0, 0.0, -10.0}, {0.707, -1.0, 0.0, -10.0},
                                       {-0.707, 0.0, 1.0, -10.0}, {-0.707, 0.0, -1.0, -10.0}};
    for (int k = 0; k < 4; ++k)
        for (int q = 0; q < 4; ++q) cont[NC + k].Ai[q] = bound[k][q];

    get_firstvert(S->seed, cont, &pA, &pB, &pC, NC, az);
    double tmp[3];
    fxo_solve_3x3(cont[pA].Ai, cont[pB].Ai, cont[pC].Ai, tmp);
    add_vertex(poly, 0, tmp, pA, pB, pC);
    cont[pA].flag = 'Y';
    cont[pB].flag = 'Y';
    cont[pC].flag = 'Y';
    add_vedge(ve, 0, cont, pA, pB, pC, poly, 0);
    add_vedge(ve, 1, cont, pB, pC, pA, poly, 0);
    add_vedge(ve, 2, cont, pC, pA, pB, poly, 0);
    int startedge = 0, edgenum = 3, vn = 1;
    const double rr = rado * rado;   /* float product, compared in double */

    for (;;) {
        while (ve[startedge].endpt >= 0 && (edgenum - startedge) > 0) ++startedge;
        if ((edgenum - startedge) <= 0) break;
        double vtmin = 9.9e+9;
        const Vert* vs = &poly[ve[startedge].startpt];
        const double* V = ve[startedge].V;
        pA = ve[startedge].plane[0];
        pB = ve[startedge].plane[1];
        oldC = ve[startedge].startplane;
        pC = -1;
        for (int c = 0; c < NC; ++c) {
            if (c != pA && c != pB && c != oldC) {
                double den = cont[c].Ai[0] * V[0] + cont[c].Ai[1] * V[1] + cont[c].Ai[2] * V[2];
                if (den != 0.0) {
                    double vt = -(cont[c].Ai[0] * vs->xi[0] + cont[c].Ai[1] * vs->xi[1] + cont[c].Ai[2] * vs->xi[2] + cont[c].Ai[3]) / den;
                    if (vt < vtmin && vt > 0) {
                        vtmin = vt;
                        pC = c;
                    }
                }
            }
        }
        poly[vn].xi[0] = vs->xi[0] + vtmin * V[0];
        poly[vn].xi[1] = vs->xi[1] + vtmin * V[1];
        poly[vn].xi[2] = vs->xi[2] + vtmin * V[2];
        if ((poly[vn].xi[0] * poly[vn].xi[0] + poly[vn].xi[1] * poly[vn].xi[1] + poly[vn].xi[2] * poly[vn].xi[2]) > rr) {
            for (int c = NC; c < NC + 4; ++c) {
                if (c != pA && c != pB && c != oldC) {
                    double den = cont[c].Ai[0] * V[0] + cont[c].Ai[1] * V[1] + cont[c].Ai[2] * V[2];
                    if (den != 0.0) {
                        double vt = -(cont[c].Ai[0] * vs->xi[0] + cont[c].Ai[1] * vs->xi[1] + cont[c].Ai[2] * vs->xi[2] + cont[c].Ai[3]) / den;
                        if (vt < vtmin && vt > 0) {
                            vtmin = vt;
                            pC = c;
                        }
                    }
                }
            }
            poly[vn].xi[0] = vs->xi[0] + vtmin * V[0];
            poly[vn].xi[1] = vs->xi[1] + vtmin * V[1];
            poly[vn].xi[2] = vs->xi[2] + vtmin * V[2];
        }
        if (pC < 0) return -1;   /* no closing plane: the reference would index cont[-1] */
        double x[3] = {poly[vn].xi[0], poly[vn].xi[1], poly[vn].xi[2]};
        add_vertex(poly, vn, x, pA, pB, pC);
        ve[startedge].endpt = vn;
        ve[startedge].endplane = pC;
        cont[pC].flag = 'Y';

        int found = 0;
        for (int ei = startedge + 1; ei < edgenum; ++ei) {
            if ((ve[ei].plane[0] == pA && ve[ei].plane[1] == pC) || (ve[ei].plane[0] == pC && ve[ei].plane[1] == pA)) {
                ve[ei].endpt = vn;
                ve[ei].endplane = pB;
                found = 1;
                break;
            }
        }
        if (!found) {
            add_vedge(ve, edgenum, cont, pA, pC, pB, poly, vn);
            ++edgenum;
        }
        found = 0;
        for (int ei = startedge + 1; ei < edgenum; ++ei) {
            if ((ve[ei].plane[0] == pB && ve[ei].plane[1] == pC) || (ve[ei].plane[0] == pC && ve[ei].plane[1] == pB)) {
                ve[ei].endpt = vn;
                ve[ei].endplane = pA;
                found = 1;
                break;
            }
        }
        if (!found) {
            add_vedge(ve, edgenum, cont, pB, pC, pA, poly, vn);
            ++edgenum;
            if (edgenum >= O_MAX_EDGES) return -1;
        }
        ++vn;
        if (vn >= O_MAX_POLY - 4 || edgenum >= O_MAX_POLY - 4) return -1;
    }
    if (S->counts) {
        S->counts->edges += edgenum;
        S->counts->plane_tests += (int64_t)edgenum * NC;
    }

    for (int ei = 0; ei < edgenum; ++ei) {
        if ((rado < poly[ve[ei].startpt].dist) || (rado < poly[ve[ei].endpt].dist)) ve[ei].arc = '?';
        else ve[ei].arc = 'X';
    }
    double a0[3], a1[3];
    for (int ei = 0; ei < edgenum; ++ei) {
        if (ve[ei].arc == 'X') continue;
        if (S->counts) S->counts->arc_edges++;
        if (fxo_solve_2xS(cont[ve[ei].plane[0]].Ai, cont[ve[ei].plane[1]].Ai, rado, a0, a1) == -1) {
            ve[ei].arc = 'X';
            continue;
        }
        const int ta = ve[ei].startplane, tb = ve[ei].endplane;
        double va = cont[ta].Ai[0] * a0[0] + cont[ta].Ai[1] * a0[1] + cont[ta].Ai[2] * a0[2] + cont[ta].Ai[3];
        double vb = cont[tb].Ai[0] * a0[0] + cont[tb].Ai[1] * a0[1] + cont[tb].Ai[2] * a0[2] + cont[tb].Ai[3];
        if (va < 0.0 && vb < 0.0) {
            add_vertex(poly, vn, a0, ve[ei].plane[0], ve[ei].plane[1], -1);
            poly[vn].dist = rado;
            ++vn;
        }
        va = cont[ta].Ai[0] * a1[0] + cont[ta].Ai[1] * a1[1] + cont[ta].Ai[2] * a1[2] + cont[ta].Ai[3];
        vb = cont[tb].Ai[0] * a1[0] + cont[tb].Ai[1] * a1[1] + cont[tb].Ai[2] * a1[2] + cont[tb].Ai[3];
        if (va < 0.0 && vb < 0.0) {
            add_vertex(poly, vn, a1, ve[ei].plane[0], ve[ei].plane[1], -1);
            poly[vn].dist = rado;
            ++vn;
        }
        if (vn >= O_MAX_POLY - 2) return -1;
    }
    int vj = 0;
    for (int vi = 0; vi < vn; ++vi)
        if (poly[vi].dist <= rado) poly[vj++] = poly[vi];
    vn = vj;
    for (int c = 0; c < NC; ++c) {
        S->centerpt[c].xi[0] = -cont[c].Ai[0] * cont[c].Ai[3];
        S->centerpt[c].xi[1] = -cont[c].Ai[1] * cont[c].Ai[3];
        S->centerpt[c].xi[2] = -cont[c].Ai[2] * cont[c].Ai[3];
        S->centerpt[c].dist = fabs(cont[c].Ai[3]);
        if (cont[c].Ai[3] > 0.0) cont[c].flag = 'E';
    }
    save_seeds(S->seed, cont, poly, vn, az);
    return vn;
}

/* First position 1..n-1 of the face list whose vertex lies on plane pY (n if none). */
static int find_partner(const Vert* poly, const int* pt, int n, int pY) {
    int vi;
    for (vi = 1; vi < n; ++vi) {
        const Vert* p = &poly[pt[vi]];
        if (p->plane[0] == pY || p->plane[1] == pY || p->plane[2] == pY) break;
    }
    return vi;
}

/* order_faces, LIB/Vcontacts.cpp:699-831: per contact plane, the polygon's vertices in
 * angular order (plus an antipodal arc point so no arc exceeds 180 degrees). */
static void order_faces(State* S, float rado, int NC, int NV) {
    Vert* poly = S->poly;
    const Plane* cont = S->cont;
    PtOrder* po = S->ptorder;
    double cos10X[O_MAX_CONT];
    for (int X = 0; X < NC; ++X) {
        if (cont[X].flag == 'X') {
            po[X].numpts = 0;
            continue;
        }
        int sc = 0;
        for (int vi = 0; vi < NV; ++vi)
            if ((poly[vi].plane[0] == X || poly[vi].plane[1] == X || poly[vi].plane[2] == X) && sc < O_MAX_CONT)
                po[X].pt[sc++] = vi;
        if (sc > 2) {
            for (int vi = 0; vi < sc; ++vi) {
                if (poly[po[X].pt[vi]].plane[2] == -1) {
                    double t[3];
                    t[0] = 2.0 * S->centerpt[X].xi[0] - poly[po[X].pt[vi]].xi[0];
                    t[1] = 2.0 * S->centerpt[X].xi[1] - poly[po[X].pt[vi]].xi[1];
                    t[2] = 2.0 * S->centerpt[X].xi[2] - poly[po[X].pt[vi]].xi[2];
                    if (test_point(t, cont, NC, X, -1, -1) == 'Y' && sc < O_MAX_CONT && NV < O_MAX_POLY) {
                        poly[NV].xi[0] = t[0];
                        poly[NV].xi[1] = t[1];
                        poly[NV].xi[2] = t[2];
                        poly[NV].plane[0] = X;
                        poly[NV].plane[1] = -1;
                        poly[NV].plane[2] = -1;
                        poly[NV].dist = rado;
                        po[X].pt[sc++] = NV;
                        ++NV;
                    }
                    break;
                }
            }
        }
        po[X].numpts = sc;
        if (sc > 3) {
            const Vert* p0 = &poly[po[X].pt[0]];
            int pY = (p0->plane[0] == X) ? p0->plane[1] : p0->plane[0];
            int vi = find_partner(poly, po[X].pt, sc, pY);
            if (vi == sc) {
                if (S->counts) S->counts->no_partner++;
                /* No vertex shares pt[0]'s second plane. The reference then swaps pt[1] with
                   the slot past the face's end, which holds whatever an earlier face left
                   there. Reference-compat mode replays that read (on a workspace zeroed at the
                   start of every pose, as the test harness arranges). By default pt[0]'s other
                   plane is tried instead, so that pt[0] and pt[1] are still neighbours on the
                   face and the angular sort orders the face's points correctly. */
                if (g_compat) {
                    if (sc >= O_MAX_CONT) vi = 1;
                } else {
                    int pZ = (p0->plane[0] == X || p0->plane[1] == X) ? p0->plane[2] : p0->plane[1];
                    if (p0->plane[0] != X && p0->plane[1] != X) pZ = p0->plane[1];
                    vi = pZ >= 0 ? find_partner(poly, po[X].pt, sc, pZ) : sc;
                    if (vi == sc) vi = 1;
                }
            }
            {
                int t = po[X].pt[vi];
                po[X].pt[vi] = po[X].pt[1];
                po[X].pt[1] = t;
            }
            for (vi = 2; vi < sc; ++vi)
                cos10X[vi] = fxo_cosPQR(poly[po[X].pt[1]].xi, poly[po[X].pt[0]].xi, poly[po[X].pt[vi]].xi);
            for (vi = 2; vi < sc - 1; ++vi)
                for (int v2 = vi + 1; v2 < sc; ++v2)
                    if (cos10X[vi] < cos10X[v2]) {
                        int t = po[X].pt[vi];
                        po[X].pt[vi] = po[X].pt[v2];
                        po[X].pt[v2] = t;
                        double tc = cos10X[vi];
                        cos10X[vi] = cos10X[v2];
                        cos10X[v2] = tc;
                    }
        }
    }
}

/* project_points, LIB/Vcontacts.cpp:1278-1344: engulfing-plane correction, projects polyhedron
 * vertices onto the sphere from the engulfing contact's centre. */
static void project_points(State* S, float rado, int NC, int NV, int az) {
    Vert* poly = S->poly;
    const Plane* cont = S->cont;
    int epi = 0, eng[4];
    for (int c = 0; c < NC; ++c)
        if (cont[c].flag == 'E') {
            eng[epi++] = c;
            if (epi == 3) break;
        }
    double pp[3], p0[3], p1[3];
    if (epi == 1) {
        pp[0] = S->centerpt[eng[0]].xi[0];
        pp[1] = S->centerpt[eng[0]].xi[1];
        pp[2] = S->centerpt[eng[0]].xi[2];
    } else if (epi == 2) {
        if (fxo_solve_2xS(cont[eng[0]].Ai, cont[eng[1]].Ai, rado, p0, p1) == -1) {
            pp[0] = S->xyz[az][0] + rado;
            pp[1] = S->xyz[az][1];
            pp[2] = S->xyz[az][2];
        } else {
            pp[0] = (p0[0] + p1[0]) / 2;
            pp[1] = (p0[1] + p1[1]) / 2;
            pp[2] = (p0[2] + p1[2]) / 2;
        }
    } else {
        fxo_solve_3x3(cont[eng[0]].Ai, cont[eng[1]].Ai, cont[eng[2]].Ai, p0);
        pp[0] = p0[0];
        pp[1] = p0[1];
        pp[2] = p0[2];
    }
    for (int vi = 0; vi < NV; ++vi) {
        if (poly[vi].plane[2] == -1) continue;
        double* P = poly[vi].xi;
        double V[3] = {P[0] - pp[0], P[1] - pp[1], P[2] - pp[2]};
        double a = V[0] * V[0] + V[1] * V[1] + V[2] * V[2];
        double b = 2 * (P[0] * V[0] + P[1] * V[1] + P[2] * V[2]);
        double c = P[0] * P[0] + P[1] * P[1] + P[2] * P[2] - rado * rado;
        double k = (sqrt(b * b - 4.0 * a * c) - b) / (2 * a);
        P[0] += k * V[0];
        P[1] += k * V[1];
        P[2] += k * V[2];
        poly[vi].dist = rado;
    }
}

/* calc_areas, LIB/Vcontacts.cpp:838-1044: spherical area of every contact face, with the
 * engulfing-plane corrections. */
static void calc_areas(State* S, float rado, int NC, int NV, int az) {
    Vert* poly = S->poly;
    Plane* cont = S->cont;
    const Vert* cp = S->centerpt;
    const PtOrder* po = S->ptorder;
    char engflag = 'N';
    int epi = 0, eng[4];
    double cosNN1[O_MAX_CONT], cosN0[O_MAX_CONT];
    for (int X = 0; X < NC; ++X) {
        cont[X].area = 0.0;
        if (cont[X].flag == 'E') {
            engflag = 'Y';
            eng[epi++] = X;
            if (epi == 3) break;
        }
    }
    if (engflag == 'Y') project_points(S, rado, NC, NV, az);
    for (int X = 0; X < NC; ++X) {
        const int NP = po[X].numpts;
        double area = 0.0;
        if (cont[X].flag == 'X') continue;
        if (NP == 0) {
            if (test_point(cp[X].xi, cont, NC, X, -1, -1) == 'Y')
                cont[X].area = 2.0f * O_PI * rado * (rado - cp[X].dist);
        } else if (NP == 2) {
            if (S->counts) S->counts->triangles++;
            if (test_point(cp[X].xi, cont, NC, X, -1, -1) == 'Y')
                cont[X].area = 2.0f * O_PI * rado * (rado - cp[X].dist) -
                               sph_arc(&cp[X], &poly[po[X].pt[0]], &poly[po[X].pt[1]], rado);
            else
                cont[X].area = sph_arc(&cp[X], &poly[po[X].pt[0]], &poly[po[X].pt[1]], rado);
        } else {
            for (int vi = 0; vi < NP; ++vi) {
                const int v0 = po[X].pt[0], va = po[X].pt[vi], vb = po[X].pt[(vi + 1) % NP];
                cosNN1[vi] = ((poly[va].xi[0] * poly[vb].xi[0] + poly[va].xi[1] * poly[vb].xi[1] + poly[va].xi[2] * poly[vb].xi[2]) /
                              (poly[va].dist * poly[vb].dist));
                if (vi != 0)
                    cosN0[vi] = ((poly[v0].xi[0] * poly[va].xi[0] + poly[v0].xi[1] * poly[va].xi[1] + poly[v0].xi[2] * poly[va].xi[2]) /
                                 (poly[v0].dist * poly[va].dist));
            }
            for (int vi = 1; vi < NP - 1; ++vi) {
                if (S->counts) S->counts->triangles++;
                double U = sqrt((1 + cosN0[vi]) * (1 + cosNN1[vi]) * (1 + cosN0[vi + 1]) / 8.0);
                double V = sqrt((1 - cosN0[vi]) * (1 - cosNN1[vi]) * (1 + cosN0[vi + 1]) / 8.0);
                double W = sqrt((1 - cosN0[vi]) * (1 + cosNN1[vi]) * (1 - cosN0[vi + 1]) / 8.0);
                double Xv = sqrt((1 + cosN0[vi]) * (1 - cosNN1[vi]) * (1 - cosN0[vi + 1]) / 8.0);
                double tS = (1 - U + V + W + Xv) / (1 + U - V - W - Xv);
                double tSA = (1 - U - V - W + Xv) / (1 + U + V + W - Xv);
                double tSB = (1 - U - V + W - Xv) / (1 + U + V - W + Xv);
                double tSC = (1 - U + V - W - Xv) / (1 + U - V + W + Xv);
                double tanprod = sqrt(tS * tSA * tSB * tSC);
                if (tanprod > 0.0) area += 4.0 * rado * rado * atan(sqrt(tanprod));
            }
            for (int vi = 0; vi < NP; ++vi) {
                const int va = po[X].pt[vi], vb = po[X].pt[(vi + 1) % NP];
                if (poly[va].plane[2] == -1 && poly[vb].plane[2] == -1) {
                    if ((poly[va].plane[0] + poly[va].plane[1]) != (poly[vb].plane[0] + poly[vb].plane[1])) {
                        if (S->counts) S->counts->triangles++;
                        area += sph_arc(&cp[X], &poly[va], &poly[vb], rado);
                    }
                }
            }
            cont[X].area = area;
        }
    }
    if (engflag != 'Y') return;
    for (int X = 0; X < NC; ++X) {
        if (cont[X].flag != 'E') continue;
        const int NP = po[X].numpts;
        for (int vi = 0; vi < NP; ++vi) {
            const int cur = po[X].pt[vi], nxt = po[X].pt[(vi + 1) % NP];
            int pa1, pa2, comm;
            if (poly[cur].plane[0] == X) {
                pa1 = poly[cur].plane[1];
                pa2 = poly[cur].plane[2];
            } else {
                pa1 = poly[cur].plane[0];
                pa2 = (poly[cur].plane[1] == X) ? poly[cur].plane[2] : poly[cur].plane[1];
            }
            if (pa1 == poly[nxt].plane[0] || pa1 == poly[nxt].plane[1] || pa1 == poly[nxt].plane[2]) comm = pa1;
            else if (pa2 == poly[nxt].plane[0] || pa2 == poly[nxt].plane[1] || pa2 == poly[nxt].plane[2]) comm = pa2;
            else continue;
            if (comm != -1 && cont[comm].flag != 'E') {
                cont[comm].area += sph_arc(&cp[X], &poly[cur], &poly[nxt], rado);
                if (NP == 2) break;
            }
        }
    }
    if (epi == 1) {
        cont[eng[0]].area = 2.0f * O_PI * rado * (rado + cont[eng[0]].dist);
    } else if (epi == 2) {
        Vert B, Cc;
        if (fxo_solve_2xS(cont[eng[0]].Ai, cont[eng[1]].Ai, rado, B.xi, Cc.xi) == -1) {
            cont[eng[0]].area = 2.0f * O_PI * rado * rado;
            cont[eng[1]].area = 2.0f * O_PI * rado * rado;
        } else {
            B.dist = rado;
            Cc.dist = rado;
            double m = sph_arc(&cp[eng[0]], &B, &Cc, rado);
            m += sph_arc(&cp[eng[1]], &B, &Cc, rado);
            cont[eng[0]].area = 2.0f * O_PI * rado * rado - 0.5 * m;
            cont[eng[1]].area = 2.0f * O_PI * rado * rado - 0.5 * m;
        }
    } else if (epi >= 3) {
        for (int X = 0; X < NC; ++X) {
            if (cont[X].flag == 'E') cont[X].area = 4.0f * O_PI * rado * rado / epi;
            else cont[X].area = 0.0f;
        }
    }
}

/* save_areas, LIB/Vcontacts.cpp:1149-1220: records the atom's contacts (reusing the stub
 * records other atoms left for it), marks it done and leaves stubs for its partners. */
static int grow_carec(State* S) {
    if (S->ncarec > S->carec_cap - 100) {
        int cap = S->carec_cap + 10000;
        CaRec* p = (CaRec*)realloc(S->carec, (size_t)cap * sizeof(CaRec));
        if (!p) return -1;
        S->carec = p;
        S->carec_cap = cap;
    }
    return 0;
}

static int save_areas(State* S, int NC, int az) {
    if (grow_carec(S)) return -1;
    const Plane* cont = S->cont;
    int c = 0, cur = S->ca_index[az], prev = -1;
    while (cur != -1 && c < NC) {
        if (cont[c].area > 0.0 && cont[c].flag != 'X') {
            S->carec[cur].from = az;
            S->carec[cur].atom = cont[c].index;
            S->carec[cur].area = cont[c].area;
            S->carec[cur].dist = S->cand[c].dist;
            int nxt = S->carec[cur].prev;
            S->carec[cur].prev = prev;
            prev = cur;
            cur = nxt;
        }
        ++c;
    }
    S->ca_index[az] = prev;
    for (; c < NC; ++c) {
        if (cont[c].area > 0.0 && cont[c].flag != 'X') {
            if (S->ncarec >= S->carec_cap && grow_carec(S)) return -1;
            CaRec* r = &S->carec[S->ncarec];
            r->from = az;
            r->atom = cont[c].index;
            r->area = cont[c].area;
            r->dist = S->cand[c].dist;
            r->prev = S->ca_index[az];
            S->ca_index[az] = S->ncarec++;
        }
    }
    S->done[az] = 'Y';
    for (c = 0; c < NC; ++c) {
        const int j = cont[c].index;
        if (S->done[j] != 'Y' && cont[c].area > 0.0 && cont[c].flag != 'X') {
            if (S->ncarec >= S->carec_cap - 1 && grow_carec(S)) return -1;
            CaRec* r = &S->carec[S->ncarec];
            r->from = j;
            r->atom = az;
            r->prev = S->ca_index[j];
            S->ca_index[j] = S->ncarec++;
        }
    }
    return 0;
}

/* residue.bonded of two Calc slots of one residue (ligand or flexible side chain); -1 when they
 * belong to different residues or are more than bloops bonds apart. */
static int residue_bonded(const State* S, const fxe_ligand_desc* lig, int a, int b) {
    const int ra = S->res_of[a];
    if (ra < 0 || ra != S->res_of[b]) return -1;
    if (ra == S->nflex) return lig->bonded[S->loc[a] * lig->n_atoms + S->loc[b]];
    const fxe_flex_residue* f = &S->flex[ra];
    return f->bonded[S->loc[a] * f->n_atoms + S->loc[b]];
}

/* get_contlist4, LIB/Vcontacts.cpp:1725-1839: atoms of the 27 surrounding cells within
 * rado + r_j + Rw, skipping atoms already done unless they recorded a contact with this one.
 * With clash != NULL it also accumulates the wall term of the pre-filter. */
static int get_contlist(State* S, const fxe_ligand_desc* lig, int az, float rado, double* clash,
                        double permea) {
    int NC = 0;
    const int dim = S->dim, dim2 = dim * dim, dim3 = dim * dim * dim;
    for (int cur = S->ca_index[az]; cur != -1; cur = S->carec[cur].prev) S->done[S->carec[cur].atom] = 'C';
    const int box0 = S->boxnum[az];
    const float* a = S->xyz[az];
    for (int i = 0; i < 27; ++i) {
        const int bi = box0 + dim2 * ((i / 9) - 1) + dim * (((i / 3) % 3) - 1) + (i % 3) - 1;
        if (bi < 0 || bi >= dim3) continue;
        for (int k = 0; k < S->box_n[bi]; ++k) {
            const int j = S->calclist[S->box_f[bi] + k];
            if (S->counts && !clash) S->counts->candidates++;
            if (S->done[j] == 'Y') continue;
            const double rAB = S->rad_all[az] + S->rad_all[j];
            const float* b = S->xyz[j];
            const double sq = (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]);
            const double nd = rado + S->rad_all[j] + O_RW;
            const double cd = permea * rAB;
            if (sq < nd * nd && sq != 0.0) {
                S->cand[NC].index = j;
                S->cand[NC].dist = sqrt(sq);
                if (clash) {
                    if (S->cand[NC].dist < cd) {
                        if (residue_bonded(S, lig, az, j) < 0)
                            *clash += O_KWALL * (pow(S->cand[NC].dist, -12.0) - pow(cd, -12.0));
                    }
                    S->done[az] = 'Y';
                }
                ++NC;
            }
        }
    }
    for (int cur = S->ca_index[az]; cur != -1; cur = S->carec[cur].prev) S->done[S->carec[cur].atom] = 'Y';
    return NC;
}

/* index_protein, LIB/Vcontacts.cpp:1570-1715, in the state after the first evaluation: the
 * receptor atoms keep their place while the scorable atoms (ligand and side-chain atoms, whose
 * Calc slots are refilled every call) are re-examined. */
static int index_atoms(State* S, const fxe_receptor_desc* rec) {
    float gmin[3], gmax[3];
    int alter = 0;
    for (int j = 0; j < 3; ++j) {
        gmin[j] = (int)rec->globalmin[j] + 1.0;
        gmax[j] = (int)rec->globalmax[j] + 1.0;
    }
    float mw = rec->maxwidth;
    for (int i = 0; i < S->natoms; ++i)
        for (int j = 0; j < 3 && S->score[i]; ++j) {
            if (S->xyz[i][j] < gmin[j]) {
                gmin[j] = S->xyz[i][j];
                alter = 1;
            } else if (S->xyz[i][j] > gmax[j]) {
                gmax[j] = S->xyz[i][j];
                alter = 1;
            }
        }
    if (alter) {
        for (int j = 0; j < 3; ++j) {
            gmin[j] = gmin[j] < 0.0 ? (int)gmin[j] - 1.0 : (int)gmin[j] + 1.0;
            gmax[j] = gmax[j] < 0.0 ? (int)gmax[j] - 1.0 : (int)gmax[j] + 1.0;
            float diff = gmax[j] - gmin[j];
            if (diff > mw) mw = diff;
        }
    }
    const int dim = (int)(mw / O_CELL) + 1;
    const int dim2 = dim * dim, dim3 = dim2 * dim;
    S->dim = dim;
    if (dim3 > S->box_cap) {
        free(S->box_n);
        free(S->box_f);
        S->box_n = (int*)malloc((size_t)dim3 * sizeof(int));
        S->box_f = (int*)malloc((size_t)dim3 * sizeof(int));
        if (!S->box_n || !S->box_f) return -1;
        S->box_cap = dim3;
    }
    memset(S->box_n, 0, (size_t)dim3 * sizeof(int));
    for (int i = 0; i < S->natoms; ++i) {
        const int bi = (int)((S->xyz[i][0] - gmin[0]) / O_CELL) * dim2 + (int)((S->xyz[i][1] - gmin[1]) / O_CELL) * dim +
                       (int)((S->xyz[i][2] - gmin[2]) / O_CELL);
        if (bi < 0 || bi >= dim3) return -2;
        S->boxnum[i] = bi;
        ++S->box_n[bi];
    }
    int st = 0;
    for (int b = 0; b < dim3; ++b) {
        S->box_f[b] = st;
        st += S->box_n[b];
        S->box_n[b] = 0;
    }
    for (int i = 0; i < S->natoms; ++i) {
        const int b = S->boxnum[i];
        S->calclist[S->box_f[b] + S->box_n[b]] = i;
        ++S->box_n[b];
    }
    return 0;
}

/* Vcontacts + calc_region, LIB/Vcontacts.cpp:6-139. Returns 0, -1 (hull failure) or -2
 * (clash pre-filter). */
static int vcontacts(State* S, const fxe_receptor_desc* rec, const fxe_ligand_desc* lig,
                     double* clash, double permea, int* err) {
    int r = index_atoms(S, rec);
    if (r) {
        *err = r;
        return -3;
    }
    for (int i = 0; i < S->natoms; ++i) {
        S->ca_index[i] = -1;
        S->seed[i * 3] = -1;
    }
    *clash = 0.0;
    for (int i = 0; i < S->natoms; ++i) {
        const int az = S->calclist[i];
        if (!S->score[az]) continue;
        const float rado = S->rad_all[az] + O_RW;
        get_contlist(S, lig, az, rado, clash, permea);
    }
    if (*clash >= O_CLASH_THRESHOLD) return -2;
    for (int i = 0; i < S->natoms; ++i) {
        S->done[i] = 'N';
        S->ca_index[i] = -1;
        S->seed[i * 3] = -1;
    }
    S->ncarec = 0;
    for (int i = 0; i < S->natoms; ++i) {
        const int az = S->calclist[i];
        if (!S->score[az]) continue;
        const float rado = S->rad_all[az] + O_RW;
        const int NC = get_contlist(S, lig, az, rado, NULL, 0.0);
        if (S->counts) {
            S->counts->atoms++;
            S->counts->contacts += NC;
        }
        if (NC == 0) continue;
        const int NV = voronoi_poly2(S, az, rado, NC);
        if (NV == -1) return -1;
        if (S->counts) S->counts->vertices += NV;
        order_faces(S, rado, NC, NV);
        calc_areas(S, rado, NC, NV, az);
        if (save_areas(S, NC, az)) {
            *err = -1;
            return -3;
        }
    }
    return 0;
}

/* ----------------------------------------------------------------------------------------
 * pose build (ic2cf IC assignment + buildcc)
 * -------------------------------------------------------------------------------------- */

/* buildcc, LIB/buildcc.cpp:6-134: Cartesian position of each atom of the rebuild list from its
 * distance, angle and dihedral to its three reference atoms (FA->ori-based points stand in for
 * missing references). Single precision throughout, as in the reference. */
static void buildcc(State* S, const fxe_receptor_desc* rec, const fxe_ligand_desc* lig) {
    const float* ori = rec->ori;
    for (int an = 0; an < lig->n_build; ++an) {
        const int l = lig->build_order[an];
        float x[4], y[4], z[4];
        for (int i = 1; i <= 3; ++i) {
            const int j = lig->rec[l * 4 + i - 1];
            if (j >= 0) {
                x[i] = S->xyz[S->nrec + j][0];
                y[i] = S->xyz[S->nrec + j][1];
                z[i] = S->xyz[S->nrec + j][2];
            } else if (i == 1) {
                x[i] = 1.0f + ori[0];
                y[i] = 0.0f + ori[1];
                z[i] = 0.0f + ori[2];
            } else if (i == 3) {
                x[i] = 0.0f + ori[0];
                y[i] = 1.0f + ori[1];
                z[i] = 0.0f + ori[2];
            } else {
                x[i] = 0.0f + ori[0];
                y[i] = 0.0f + ori[1];
                z[i] = 0.0f + ori[2];
            }
            x[i] += 1e-10f;
            y[i] += 1e-10f;
            z[i] += 1e-10f;
        }
        float a = y[1] * (z[2] - z[3]) + y[2] * (z[3] - z[1]) + y[3] * (z[1] - z[2]);
        float b = z[1] * (x[2] - x[3]) + z[2] * (x[3] - x[1]) + z[3] * (x[1] - x[2]);
        float c = x[1] * (y[2] - y[3]) + x[2] * (y[3] - y[1]) + x[3] * (y[1] - y[2]);
        float op = sqrtf(a * a + b * b + c * c);
        float cx = a / op, cy = b / op, cz = c / op;
        a = x[2] - x[1];
        b = y[2] - y[1];
        c = z[2] - z[1];
        float d = 1.0f / sqrtf(a * a + b * b + c * c);
        op = S->lic[l][0] * d;
        float xn = a * op, yn = b * op, zn = c * op;
        a = cx * cx;
        b = cy * cy;
        c = cz * cz;
        float angPI = (float)(S->lic[l][1] * O_PI / 180.0f);
        float ct = o_cosf(angPI), st = -o_sinf(angPI);
        op = 1.0f - ct;
        float xk = (cx * cz * op - cy * st) * zn + ((1.0f - a) * ct + a) * xn + (cx * cy * op + cz * st) * yn;
        float yk = (cy * cx * op - cz * st) * xn + ((1.0f - b) * ct + b) * yn + (cy * cz * op + cx * st) * zn;
        float zk = (cz * cy * op - cx * st) * yn + ((1.0f - c) * ct + c) * zn + (cz * cx * op + cy * st) * xn;
        float dihPI = (float)(S->lic[l][2] * O_PI / 180.0f);
        ct = o_cosf(dihPI);
        st = o_sinf(dihPI);
        op = 1.0f - ct;
        cx = (x[2] - x[1]) * d;
        cy = (y[2] - y[1]) * d;
        cz = (z[2] - z[1]) * d;
        a = cx * cx;
        b = cy * cy;
        c = cz * cz;
        float* o = S->xyz[S->nrec + l];
        o[0] = (cx * cz * op - cy * st) * zk + ((1.0f - a) * ct + a) * xk + (cx * cy * op + cz * st) * yk + x[1];
        o[1] = (cy * cx * op - cz * st) * xk + ((1.0f - b) * ct + b) * yk + (cy * cz * op + cx * st) * zk + y[1];
        o[2] = (cz * cy * op - cx * st) * yk + ((1.0f - c) * ct + c) * zk + (cz * cx * op + cy * st) * xk + z[1];
        if (S->counts) S->counts->built_atoms++;
    }
}

/* IC assignment of ic2cf, LIB/ic2cf.cpp:53-105 (grid index, angle, dihedral with the rec[3]
 * cascade). */
static void assign_ic(State* S, const fxe_receptor_desc* rec, const fxe_ligand_desc* lig,
                      const double* icv) {
    for (int l = 0; l < lig->n_atoms; ++l)
        for (int k = 0; k < 3; ++k) S->lic[l][k] = lig->ic[l * 3 + k];
    for (int g = 0; g < lig->n_genes; ++g) {
        const int atm = lig->gene_atom[g];
        switch (lig->gene_type[g]) {
        case -1: {
            const unsigned gi = (unsigned)icv[g];
            S->lic[atm][0] = rec->grid_ic[gi * 3 + 0];
            S->lic[atm][1] = rec->grid_ic[gi * 3 + 1];
            S->lic[atm][2] = rec->grid_ic[gi * 3 + 2];
            break;
        }
        case 0: S->lic[atm][0] = (float)icv[g]; break;
        case 1: S->lic[atm][1] = (float)icv[g]; break;
        case 2: {
            S->lic[atm][2] = (float)icv[g];
            int j = atm, cat = lig->rec[atm * 4 + 3];
            if (cat >= 0) {
                int guard = 0;
                while (cat != atm && guard++ <= lig->n_atoms) {
                    S->lic[cat][2] = S->lic[j][2] + lig->shift[cat];
                    j = cat;
                    cat = lig->rec[j * 4 + 3];
                }
            }
            break;
        }
        default: break;
        }
    }
}

/* get_yval, LIB/vcfunction.cpp:576-621 */
static double get_yval(const fxe_emat_desc* em, int idx, double rel) {
    const int o = em->offset[idx], e = em->offset[idx + 1];
    if (em->weight[idx]) return em->y[o];
    int k = o;
    while (k + 1 < e && rel > em->x[k + 1]) ++k;
    if (em->x[k] > rel) return 0.0;
    if (k + 1 >= e) return em->y[k];
    return em->y[k] + (rel - em->x[k]) / (em->x[k + 1] - em->x[k]) * (em->y[k + 1] - em->y[k]);
}

/* vcfunction, LIB/vcfunction.cpp:14-574, after a successful Vcontacts: walks each scorable
 * atom's contact records in Calc order (side-chain atoms, then the ligand) and accumulates
 * com / wal / sas into its residue's record; ic2cf then adds the records up, the ligand's first
 * and the side chains' in order (LIB/ic2cf.cpp:133-245). */
static void score(State* S, const fxe_ligand_desc* lig, const fxe_emat_desc* em,
                  const fxe_params* prm, fxe_cf* cf, int pose, fxo_contact* cout, int64_t cap,
                  int64_t* ncout) {
    const int T = em->ntypes;
    const double permea = (double)prm->permeability;
    const double dee_clash = (double)prm->dee_clash;
    char* counted = (char*)calloc((size_t)S->natoms, 1);
    double rcom[O_MAX_FLEX + 1] = {0}, rwal[O_MAX_FLEX + 1] = {0}, rsas[O_MAX_FLEX + 1] = {0};
    double totsas = 0.0;
    int rclash = 0;
    for (int i = 0; i < S->natoms; ++i) {
        if (!S->score[i]) continue;
        const int ri = S->res_of[i];
        const int side = ri < S->nflex;
        const double radA = (double)S->rad_all[i];
        const double radoA = radA + O_RW;
        double SAS = 4.0 * O_PI * radoA * radoA;
        const double surfA = SAS;
        for (int cur = S->ca_index[i]; cur != -1; cur = S->carec[cur].prev) {
            const int j = S->carec[cur].atom;
            const double radB = (double)S->rad_all[j];
            const double rAB = radA + radB;
            const double area = S->carec[cur].area;
            const int eidx = (S->type_all[i] - 1) * T + (S->type_all[j] - 1);
            const double yval = get_yval(em, eidx, area / surfA);
            SAS -= area;
            if (cout && *ncout < cap) {
                fxo_contact* c = &cout[*ncout];
                c->pose = pose;
                c->atom = S->mob[i];
                c->partner = j;
                c->area = (float)area;
                c->dist = (float)S->carec[cur].dist;
            }
            if (ncout) ++*ncout;
            const int same = ri == S->res_of[j];
            if (same && residue_bonded(S, lig, j, i) >= 0) continue;
            if (counted[j]) continue;
            const float clash_distance = permea * rAB;
            const double dd = S->carec[cur].dist;
            if (dd < clash_distance) {
                double d2 = dd * dd, d4 = d2 * d2, d6 = d4 * d2;
                double inv_d12 = 1.0 / (d6 * d6);
                double cr = permea * rAB;
                double cr2 = cr * cr, cr4 = cr2 * cr2, cr6 = cr4 * cr2;
                double inv_cr12 = 1.0 / (cr6 * cr6);
                rwal[ri] += O_KWALL * (inv_d12 - inv_cr12);
                if (dd <= dee_clash * rAB) rclash = 1;
            }
            /* intramolecular: one residue, or two protein residues (LIB/vcfunction.cpp:283-291) */
            const int intra = same || (side && S->res_of[j] != S->nflex);
            if (prm->intramolecular || !intra) {
                double contribution = em->weight[eidx] ? yval * area : yval;
                rcom[ri] += contribution;
            }
        }
        if (SAS < 0.0) SAS = 0.0;
        if (!side) totsas += SAS;
        double contribution;
        if (prm->solventterm) {
            contribution = (double)prm->solventterm * SAS;
        } else {
            const int eidx = (S->type_all[i] - 1) * T + (T - 1);
            const double yval = get_yval(em, eidx, SAS / surfA);
            contribution = em->weight[eidx] ? yval * SAS : yval;
        }
        rsas[ri] += contribution;
        counted[i] = 1;
    }
    free(counted);
    memset(cf, 0, sizeof(*cf));
    cf->com = 0.0 + rcom[S->nflex];
    cf->wal = 0.0 + rwal[S->nflex];
    cf->sas = 0.0 + rsas[S->nflex];
    for (int r = 0; r < S->nflex; ++r) {
        cf->com += rcom[r];
        cf->wal += rwal[r];
        cf->sas += rsas[r];
    }
    cf->con = 0.0;
    cf->totsas = totsas;
    /* ic2cf only reads the per-residue clash flag of flexible side chains; for the ligand the
       returned record keeps rclash = 0 (LIB/ic2cf.cpp:140, 150-160) */
    (void)rclash;
    cf->rclash = 0;
    cf->evalue = cf->com + cf->wal + cf->sas + cf->con + cf->elec + cf->hbond + cf->gist_desolv + cf->metal_coord;
    cf->status = FXE_POSE_SCORED;
}

/* ----------------------------------------------------------------------------------------
 * entry points
 * -------------------------------------------------------------------------------------- */

int fxo_eval_ic(const fxe_receptor_desc* rec, const fxe_ligand_desc* lig,
                const fxe_emat_desc* em, const fxe_params* prm, int32_t n, const double* ic,
                fxe_cf* out, float* xyz_out, fxo_contact* cout, int64_t cap,
                int64_t* ncout, fxo_counts* counts) {
    if (!rec || !lig || !em || !prm || n < 0 || (n > 0 && (!ic || !out))) return -1;
    State S;
    memset(&S, 0, sizeof(S));
    S.nrec = rec->n_atoms;
    S.nlig = lig->n_atoms;
    S.natoms = S.nrec + S.nlig;
    S.counts = counts;
    const int N = S.natoms;
    S.xyz = (float(*)[3])malloc((size_t)N * sizeof(*S.xyz));
    S.rad_all = (float*)malloc((size_t)N * sizeof(float));
    S.type_all = (int*)malloc((size_t)N * sizeof(int));
    S.done = (char*)malloc((size_t)N);
    S.boxnum = (int*)malloc((size_t)N * sizeof(int));
    S.calclist = (int*)malloc((size_t)N * sizeof(int));
    S.ca_index = (int*)malloc((size_t)N * sizeof(int));
    S.seed = (int*)malloc((size_t)N * 3 * sizeof(int));
    S.carec_cap = 5 * N + 200;
    S.carec = (CaRec*)malloc((size_t)S.carec_cap * sizeof(CaRec));
    S.cand = (Cand*)malloc((size_t)(N + 8) * sizeof(Cand));
    S.cont = (Plane*)malloc((size_t)(N + 8) * sizeof(Plane));
    S.centerpt = (Vert*)malloc((size_t)(N + 8) * sizeof(Vert));
    S.ptorder = (PtOrder*)calloc((size_t)(N + 8), sizeof(PtOrder));
    S.poly = (Vert*)malloc(O_MAX_POLY * sizeof(Vert));
    S.vedge = (Edge*)malloc(O_MAX_POLY * sizeof(Edge));
    S.lic = (float(*)[3])malloc((size_t)S.nlig * sizeof(*S.lic));
    S.score = (char*)calloc((size_t)N, 1);
    S.res_of = (int*)malloc((size_t)N * sizeof(int));
    S.loc = (int*)malloc((size_t)N * sizeof(int));
    S.mob = (int*)malloc((size_t)N * sizeof(int));
    S.nflex = rec->n_flex;
    S.flex = rec->flex;
    int rc = 0;
    if (!S.xyz || !S.rad_all || !S.type_all || !S.done || !S.boxnum || !S.calclist || !S.ca_index || !S.seed ||
        !S.carec || !S.cand || !S.cont || !S.centerpt || !S.ptorder || !S.poly || !S.vedge || !S.lic ||
        !S.score || !S.res_of || !S.loc || !S.mob || S.nflex < 0 || S.nflex > O_MAX_FLEX) {
        rc = -1;
        goto cleanup;
    }
    for (int i = 0; i < N; ++i) {
        S.res_of[i] = -1;
        S.loc[i] = 0;
        S.mob[i] = -1;
    }
    {
        int m = 0;
        for (int r = 0; r < S.nflex; ++r)
            for (int k = 0; k < S.flex[r].n_atoms; ++k) {
                const int i = S.flex[r].first + k;
                S.res_of[i] = r;
                S.loc[i] = k;
                if (!S.flex[r].backbone[k]) {
                    S.score[i] = 1;
                    S.mob[i] = m++;
                }
            }
        for (int l = 0; l < S.nlig; ++l) {
            S.res_of[S.nrec + l] = S.nflex;
            S.loc[S.nrec + l] = l;
            S.score[S.nrec + l] = 1;
            S.mob[S.nrec + l] = m++;
        }
    }
    for (int i = 0; i < S.nrec; ++i) {
        for (int k = 0; k < 3; ++k) S.xyz[i][k] = rec->xyz[i * 3 + k];
        S.rad_all[i] = rec->radius[i];
        S.type_all[i] = rec->type[i];
    }
    for (int l = 0; l < S.nlig; ++l) {
        S.rad_all[S.nrec + l] = lig->radius[l];
        S.type_all[S.nrec + l] = lig->type[l];
        for (int k = 0; k < 3; ++k) S.xyz[S.nrec + l][k] = 0.0f;
    }
    for (int i = 0; i < N; ++i) S.done[i] = 'N';
    if (ncout) *ncout = 0;
    double* icv = (double*)malloc((size_t)(lig->n_genes > 0 ? lig->n_genes : 1) * sizeof(double));
    for (int p = 0; p < n; ++p) {
        for (int g = 0; g < lig->n_genes; ++g) {
            double v = ic[(size_t)p * lig->n_genes + g];
            if (v > lig->gene_max[g]) v = lig->gene_max[g];
            else if (v < lig->gene_min[g]) v = lig->gene_min[g];
            icv[g] = v;
        }
        assign_ic(&S, rec, lig, icv);
        buildcc(&S, rec, lig);
        /* rotamer genes (LIB/ic2cf.cpp:90-94); index_protein refills the scored slots of the
           side chains with the selected rotamer's atoms (LIB/Vcontacts.cpp:1600-1625) */
        for (int g = 0; g < lig->n_genes; ++g) {
            if (lig->gene_type[g] != 4) continue;
            const fxe_flex_residue* f = &S.flex[lig->gene_atom[g]];
            const unsigned rot = (unsigned)(icv[g] + 0.5f);
            for (int k = 0; k < f->n_atoms; ++k) {
                if (f->backbone[k]) continue;
                for (int c = 0; c < 3; ++c) S.xyz[f->first + k][c] = f->rot_xyz[((size_t)rot * f->n_atoms + k) * 3 + c];
            }
        }
        if (xyz_out)
            for (int l = 0; l < S.nlig; ++l)
                for (int k = 0; k < 3; ++k) xyz_out[((size_t)p * S.nlig + l) * 3 + k] = S.xyz[S.nrec + l][k];
        double clash = 0.0;
        int err = 0;
        for (int i = 0; i < N; ++i)
            if (S.score[i]) S.done[i] = 'N';
        if (g_compat) memset(S.ptorder, 0, (size_t)(N + 8) * sizeof(PtOrder));
        const int rv = vcontacts(&S, rec, lig, &clash, (double)prm->permeability, &err);
        fxe_cf* cf = &out[p];
        if (rv == 0) {
            score(&S, lig, em, prm, cf, p, cout, cap, ncout);
        } else {
            memset(cf, 0, sizeof(*cf));
            if (rv == -3) {
                cf->status = FXE_POSE_CAPACITY;
                cf->evalue = 0.0;
                continue;
            }
            /* the reference's positional initialiser puts 1 into metal_coord, not rclash
               (LIB/ic2cf.cpp:127-131) */
            cf->wal = rv == -1 ? (double)O_POLY_PENALTY : clash;
            cf->metal_coord = 1.0;
            cf->rclash = 0;
            cf->evalue = cf->com + cf->wal + cf->sas + cf->con + cf->elec + cf->hbond + cf->gist_desolv + cf->metal_coord;
            cf->status = rv == -1 ? FXE_POSE_POLYHEDRON_FAILED : FXE_POSE_CLASHED;
        }
    }
    free(icv);
cleanup:
    free(S.xyz); free(S.rad_all); free(S.type_all); free(S.done); free(S.boxnum); free(S.calclist);
    free(S.ca_index); free(S.seed); free(S.carec); free(S.cand); free(S.cont); free(S.centerpt);
    free(S.ptorder); free(S.poly); free(S.vedge); free(S.lic); free(S.box_n); free(S.box_f);
    free(S.score); free(S.res_of); free(S.loc); free(S.mob);
    return rc;
}

/* genetoic with set_bins, LIB/gaboom.cpp:2887-2906 and :2295-2308. */
int fxo_genes_to_ic(const fxe_ligand_desc* lig, int32_t n, const int32_t* genes, double* ic) {
    for (int g = 0; g < lig->n_genes; ++g) {
        double nbin = (lig->gene_max[g] - lig->gene_min[g]) / lig->gene_del[g];
        if (nbin - (int)nbin > 0.0) nbin += 1.0;
        if (lig->gene_map[g]) nbin += 1.0;
        const double bin = 1.0 / nbin;
        for (int p = 0; p < n; ++p) {
            const double u = genes[(size_t)p * lig->n_genes + g] / ((double)2147483647 + 1.0);
            int i = 0;
            double tot = bin;
            while (tot < u) {
                tot += bin;
                i++;
            }
            ic[(size_t)p * lig->n_genes + g] = lig->gene_min[g] + lig->gene_del[g] * (double)i;
        }
    }
    return 0;
}

/* StatMechEngine::compute, LIB/statmech.cpp:73-174, with the max-shifted log-sum-exp of
 * LIB/UnifiedHardwareDispatch.cpp:800-843; kB = 0.001987206 kcal/mol/K (LIB/statmech.h:26). */
int fxo_thermo(const double* e, const int32_t* mult, int64_t n, double T, fxe_thermo* out) {
    if (n <= 0 || !e || !out || !(T > 0.0)) return -1;
    const double kB = 0.001987206;
    const double beta = 1.0 / (kB * T);
    double* lw = (double*)malloc((size_t)n * sizeof(double));
    if (!lw) return -1;
    double xmax = -INFINITY;
    for (int64_t i = 0; i < n; ++i) {
        lw[i] = log((double)(mult ? mult[i] : 1)) - beta * e[i];
        if (lw[i] > xmax) xmax = lw[i];
    }
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += exp(lw[i] - xmax);
    const double lnZ = xmax + log(s);
    double Ea = 0.0, E2 = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double p = exp(lw[i] - lnZ);
        Ea += p * e[i];
        E2 += p * e[i] * e[i];
    }
    free(lw);
    const double kT = kB * T;
    const double var = E2 - Ea * Ea;
    out->temperature = T;
    out->log_Z = lnZ;
    out->free_energy = -kT * lnZ;
    out->mean_energy = Ea;
    out->mean_energy_sq = E2;
    out->heat_capacity = var / (kT * kT);
    out->entropy = (Ea - out->free_energy) / T;
    out->std_energy = sqrt(var > 0.0 ? var : 0.0);
    return 0;
}

/* StatMechEngine::boltzmann_weights, LIB/statmech.cpp:178-201: normalised n_i exp(-beta E_i). */
int fxo_thermo_weights(const double* e, const int32_t* mult, int64_t n, double T, double* w) {
    if (n <= 0 || !e || !w || !(T > 0.0)) return -1;
    const double beta = 1.0 / (0.001987206 * T);
    double emin = e[0];
    for (int64_t i = 1; i < n; ++i) if (e[i] < emin) emin = e[i];
    double z = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        w[i] = (mult ? mult[i] : 1) * exp(-beta * (e[i] - emin));
        z += w[i];
    }
    for (int64_t i = 0; i < n; ++i) w[i] /= z;
    return 0;
}

/* ----------------------------------------------------------------------------------------
 * CF-based clustering (cluster, LIB/cluster.cpp:9-182)
 * -------------------------------------------------------------------------------------- */

/* Ligand coordinates of n chromosomes as calc_rmsd_chrom builds them
 * (LIB/calc_rmsd_chrom.cpp:7-145): the ICs as given (no clamp), assigned as ic2cf does, then
 * buildcc; xyz_out holds n * n_lig * 3 floats, atoms in ligand order. */
int fxo_build_ic(const fxe_receptor_desc* rec, const fxe_ligand_desc* lig, int32_t n, const double* ic,
                 float* xyz_out) {
    if (!rec || !lig || n < 0 || (n > 0 && (!ic || !xyz_out))) return -1;
    State S;
    memset(&S, 0, sizeof(S));
    S.nrec = 0;
    S.nlig = lig->n_atoms;
    S.xyz = (float(*)[3])calloc((size_t)(S.nlig > 0 ? S.nlig : 1), sizeof(*S.xyz));
    S.lic = (float(*)[3])calloc((size_t)(S.nlig > 0 ? S.nlig : 1), sizeof(*S.lic));
    if (!S.xyz || !S.lic) {
        free(S.xyz);
        free(S.lic);
        return -1;
    }
    for (int p = 0; p < n; ++p) {
        const double* icv = ic + (size_t)p * lig->n_genes;
        for (int g = 0; g < lig->n_genes; ++g)
            if (lig->gene_type[g] == -1 && !(icv[g] >= 0.0 && icv[g] < (double)rec->n_grid)) {
                free(S.xyz);
                free(S.lic);
                return -1;
            }
        assign_ic(&S, rec, lig, icv);
        buildcc(&S, rec, lig);
        for (int l = 0; l < S.nlig; ++l)
            for (int k = 0; k < 3; ++k) xyz_out[((size_t)p * S.nlig + l) * 3 + k] = S.xyz[l][k];
    }
    free(S.xyz);
    free(S.lic);
    return 0;
}

/* QuickSort_Clusters and swap_clusters, LIB/cluster.cpp:323-374 (QS_ASC(a,b) = a - b,
 * LIB/gaboom.h:40). The reference swaps its per-chromosome Clus_GAPOP entries along with the
 * cluster entries; that array is returned here as it was before the sort. */
static void qs_clusters(int* top, int* fre, double* tcf, double* acf, int beg, int end) {
    while (beg < end) {
        int l = beg, p = beg + (end - beg) / 2, r = end;
        const double piv = acf[p];
        for (;;) {
            while (l <= r && (acf[l] - piv) <= 0) ++l;
            while (l <= r && (acf[r] - piv) > 0) --r;
            if (l > r) break;
            { int t = top[l]; top[l] = top[r]; top[r] = t; t = fre[l]; fre[l] = fre[r]; fre[r] = t; }
            { double t = tcf[l]; tcf[l] = tcf[r]; tcf[r] = t; t = acf[l]; acf[l] = acf[r]; acf[r] = t; }
            if (p == r) p = l;
            ++l;
            --r;
        }
        { int t = top[p]; top[p] = top[r]; top[r] = t; t = fre[p]; fre[p] = fre[r]; fre[r] = t; }
        { double t = tcf[p]; tcf[p] = tcf[r]; tcf[r] = t; t = acf[p]; acf[p] = acf[r]; acf[r] = t; }
        --r;
        if ((r - beg) < (end - l)) {
            qs_clusters(top, fre, tcf, acf, beg, r);
            beg = l;
        } else {
            qs_clusters(top, fre, tcf, acf, l, end);
            end = r;
        }
    }
}

/* cluster, LIB/cluster.cpp:9-218: the coordinate cache, the partition function, the clusters
 * formed head by head, the ACF sort, and the RMSD between cluster heads of the .cad file
 * (calc_rmsd_chrom with calc_rmsd = true: sqrdist summed atom by atom, LIB/geometry.cpp:96-102).
 * Outputs as fxe_cluster (include/fxe.h). Returns 0, -1 on invalid input, -2 when the partition
 * function is zero (the reference stops, LIB/cluster.cpp:83-88). */
int fxo_cluster(const fxe_receptor_desc* rec, const fxe_ligand_desc* lig, int32_t n, const double* ic,
                const double* app_evalue, int32_t temperature, float rmsd_threshold, int32_t max_results,
                int32_t* top, int32_t* freq, double* tcf, double* acf, int32_t* member_of, float* rmsd,
                float* top_rmsd, int32_t* n_clusters) {
    if (!rec || !lig || n < 1 || !ic || !app_evalue || temperature < 0 || max_results < 1 || !top || !freq ||
        !tcf || !acf || !n_clusters)
        return -1;
    const int nl = lig->n_atoms, stride = 3 * nl;
    const int m = n > max_results ? n : max_results;
    float* xyz = (float*)malloc((size_t)n * stride * sizeof(float));
    int* gap = (int*)malloc((size_t)n * sizeof(int));
    float* rt = (float*)calloc((size_t)n, sizeof(float));
    double* cacf = (double*)calloc((size_t)m, sizeof(double));
    double* ctcf = (double*)calloc((size_t)m, sizeof(double));
    int* ctop = (int*)calloc((size_t)m, sizeof(int));
    int* cfre = (int*)calloc((size_t)m, sizeof(int));
    int rc = 0;
    if (!xyz || !gap || !rt || !cacf || !ctcf || !ctop || !cfre || fxo_build_ic(rec, lig, n, ic, xyz) != 0) {
        rc = -1;
        goto done;
    }
    {
        const unsigned T = (unsigned)temperature;
        const double beta = T ? (double)(1.0 / T) : 0.0;
        double pf = 0.0;
        for (int j = 0; j < n; ++j) {
            gap[j] = -1;
            if (T) pf += exp((-1.0) * beta * app_evalue[j]);
        }
        if (T && pf == 0.0) {
            rc = -2;
            goto done;
        }
        int nunc = n, nc = 0;
        while (nunc > 0) {
            int j;
            for (j = 0; j < n; ++j)
                if (gap[j] == -1) break;
            if (j >= n) break;
            gap[j] = j;
            rt[j] = 0.0f;
            nunc--;
            if (T > 0) {
                const double Pj = exp((-1.0) * beta * app_evalue[j]) / pf;
                cacf[nc] = (double)((Pj * app_evalue[j]) - (T * Pj * log(Pj)));
                ctcf[nc] = (double)((Pj * app_evalue[j]) - (T * Pj * log(Pj)));
            } else {
                ctcf[nc] = app_evalue[j];
                cacf[nc] = app_evalue[j];
            }
            ctop[nc] = j;
            cfre[nc]++;
            const float* cj = xyz + (size_t)j * stride;
            for (int i = j + 1; i < n; ++i) {
                if (gap[i] != -1) continue;
                const float* ci = xyz + (size_t)i * stride;
                /* flexaids::sum_sq_distances_f, scalar form (LIB/simd_distance.h:712-713) */
                float d = 0.0f;
                for (int k = 0; k < stride; ++k) {
                    const float t = ci[k] - cj[k];
                    d += t * t;
                }
                const float loc = sqrtf(d / (float)nl);
                if (loc <= rmsd_threshold) {
                    gap[i] = j;
                    rt[i] = loc;
                    nunc--;
                    if (T) {
                        const double Pi = exp((-1.0) * beta * app_evalue[i]) / pf;
                        cacf[nc] += (double)((Pi * app_evalue[i]) + (T * Pi * log(Pi)));
                    } else {
                        cacf[nc] += app_evalue[i];
                    }
                    cfre[nc]++;
                }
            }
            nc++;
            if (nc == max_results) break;
        }
        if (T) qs_clusters(ctop, cfre, ctcf, cacf, 0, (max_results < n ? max_results : n) - 1);
        for (int k = 0; k < max_results; ++k) {
            top[k] = ctop[k];
            freq[k] = cfre[k];
            tcf[k] = ctcf[k];
            acf[k] = cacf[k];
        }
        if (top_rmsd)
            for (int a = 0; a < max_results; ++a)
                for (int b = 0; b < max_results; ++b) {
                    const float* pa = xyz + (size_t)ctop[a] * stride;
                    const float* pb = xyz + (size_t)ctop[b] * stride;
                    float s = 0.0f;
                    for (int l = 0; l < nl; ++l) {
                        const float d0 = pa[3 * l] - pb[3 * l];
                        const float d1 = pa[3 * l + 1] - pb[3 * l + 1];
                        const float d2 = pa[3 * l + 2] - pb[3 * l + 2];
                        s += d0 * d0 + d1 * d1 + d2 * d2;
                    }
                    top_rmsd[(size_t)a * max_results + b] = (float)sqrt(s / ((float)nl));
                }
        if (member_of) memcpy(member_of, gap, (size_t)n * sizeof(int));
        if (rmsd) memcpy(rmsd, rt, (size_t)n * sizeof(float));
        *n_clusters = nc;
    }
done:
    free(xyz);
    free(gap);
    free(rt);
    free(cacf);
    free(ctcf);
    free(ctop);
    free(cfre);
    return rc;
}
