/* fvm_oracle.c -- CPU restatement of FVMR's explicit finite-volume step.
 *
 * TEST INFRASTRUCTURE ONLY (see fvm_oracle.h).  Every routine restates the
 * reference CPU path operation by operation, in the same order, so that with
 * -ffp-contract=off it reproduces the reference compiled with myfloat=double
 * bit for bit.  File:line citations are paths inside the reference project.
 */
#include "fvm_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* FVMR/src/math/CommonValue.h:16-29 */
#define OM_PI 3.1415926535897
#define OM_EPS 1e-10
#define OM_RHO_MAX 300.0
#define OM_RHO_MIN OM_EPS
#define OM_P_MAX (400.0 * 101325.0)
#define OM_P_MIN OM_EPS
/* FVMR/src/global/Constexpr.h:14-57 */
#define BC_WALL_NONVISCOUS 6001
#define BC_WALL_ADIABAT 6002
#define BC_INLET 6011
#define BC_OUTLET 6012
#define BC_INF 6013
#define BC_DSR 6014
#define BC_SYMMETRY 6021
#define BC_PERIODIC_0 6100
#define BC_PERIODIC_9 6109

/* FVMR/src/math/BasicAlgorithm.h:9-25 (argument order matters for NaN) */
static inline double m_max(double a, double b) { return (a > b) ? a : b; }
static inline double m_min(double a, double b) { return (a < b) ? a : b; }
static inline double m_abs(double a) { return (a > 0) ? a : (-a); }
static inline double m_dist2(double x1, double y1, double x2, double y2) {
    double dx = x2 - x1, dy = y2 - y1;
    return sqrt(dx * dx + dy * dy);
}

/* ------------------------------------------------------------------------ */
/* mesh reading and assembly                                                 */
/* ------------------------------------------------------------------------ */

typedef struct { int n0, n1; } om_pair;
typedef struct { char name[64]; int nedge, cap; om_pair* e; } om_marker;

typedef struct { /* open-addressing map from an unordered node pair to an edge index */
    uint64_t* key;
    int* val;
    size_t cap;
} om_emap;

static uint64_t om_key(int a, int b) {
    uint32_t lo = (uint32_t)(a < b ? a : b), hi = (uint32_t)(a < b ? b : a);
    return ((uint64_t)lo << 32) | (uint64_t)hi;
}
static size_t om_hash(uint64_t k, size_t cap) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdULL; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ULL; k ^= k >> 33;
    return (size_t)k & (cap - 1);
}
static int om_emap_get(const om_emap* h, int a, int b) {
    uint64_t k = om_key(a, b);
    for (size_t i = om_hash(k, h->cap);; i = (i + 1) & (h->cap - 1)) {
        if (h->val[i] < 0) return -1;
        if (h->key[i] == k) return h->val[i];
    }
}
static void om_emap_put(om_emap* h, int a, int b, int v) {
    uint64_t k = om_key(a, b);
    for (size_t i = om_hash(k, h->cap);; i = (i + 1) & (h->cap - 1)) {
        if (h->val[i] < 0) { h->key[i] = k; h->val[i] = v; return; }
    }
}

static void om_split(char* line, char** w, int* nw, int maxw) {
    /* StringProcessor::splitString (FVMR/src/global/StringProcessor.cpp:21-45):
     * words separated by ' ', '\t' or ','; '=' is first widened to " = "
     * (SU2MeshReader.cpp:47), which only separates it. */
    *nw = 0;
    char* s = line;
    while (*s && *nw < maxw) {
        while (*s == ' ' || *s == '\t' || *s == ',' ) s++;
        if (!*s) break;
        if (*s == '=') { w[(*nw)++] = "="; *s = 0; s++; continue; }
        w[(*nw)++] = s;
        while (*s && *s != ' ' && *s != '\t' && *s != ',' && *s != '=') s++;
        if (*s == '=') { /* keep '=' as its own word */
            *s = 0; s++;
            if (*nw < maxw) w[(*nw)++] = "=";
            continue;
        }
        if (*s) *s++ = 0;
    }
}

/* BoundaryManager::boundaryNameToType, FVMR/src/boundary_condition/BoundaryManager.cpp:15-45 */
static int om_bc_type(const char* name, int equation) {
    if (!strcmp(name, "wall") || !strcmp(name, "obstacle") || !strcmp(name, "airfoil") || !strcmp(name, "foil"))
        return equation == 1 ? BC_WALL_NONVISCOUS : BC_WALL_ADIABAT;
    if (!strcmp(name, "wall_nonViscous") || !strcmp(name, "wall_slippery") || !strcmp(name, "slippery") ||
        !strcmp(name, "slippery_wall"))
        return BC_WALL_NONVISCOUS;
    if (!strcmp(name, "inlet")) return BC_INLET;
    if (!strcmp(name, "outlet")) return BC_OUTLET;
    if (!strcmp(name, "inf") || !strcmp(name, "infinity") || !strcmp(name, "far") || !strcmp(name, "farfield"))
        return BC_INF;
    if (!strcmp(name, "dsr")) return BC_DSR;
    if (!strcmp(name, "symmetry")) return BC_SYMMETRY;
    if (!strncmp(name, "periodic", 8)) {
        size_t L = strlen(name);
        char c = name[L - 1];
        if (c < '0' || c > '9') return -2;
        return BC_PERIODIC_0 + (c - '0');
    }
    return -2;
}

#define OM_FAIL(...) do { snprintf(err, (size_t)errlen, __VA_ARGS__); goto fail; } while (0)

om_mesh* om_mesh_read_su2(const char* path, int equation, double scale, char* err, int errlen) {
    om_mesh* m = NULL;
    FILE* f = NULL;
    double *nx = NULL, *ny = NULL;
    int *nid = NULL, *tri = NULL, *idx = NULL;
    om_marker* mk = NULL;
    int nmk = 0;
    int *eL = NULL, *eR = NULL, *en0 = NULL, *en1 = NULL, *eset = NULL, *pedges = NULL;
    om_emap h = {0};
    size_t nnode = 0, capnode = 1024, ntri = 0, captri = 1024;
    int maxnodeID = 1;
    enum { S_START, S_NDIME, S_NPOIN, S_NELEM, S_NMARK } state = S_START;
    char buf[300];
    if (errlen > 0) err[0] = 0;

    f = fopen(path, "r");
    if (!f) OM_FAIL("cannot open file %s", path);
    nx = (double*)malloc(capnode * sizeof(double));
    ny = (double*)malloc(capnode * sizeof(double));
    nid = (int*)malloc(capnode * sizeof(int));
    tri = (int*)malloc(captri * 3 * sizeof(int));
    /* SU2MeshReader::readMesh, FVMR/src/input/SU2MeshReader.cpp:21-155 (lines of < 300 chars) */
    while (fgets(buf, sizeof buf, f)) {
        size_t L = strlen(buf);
        while (L && (buf[L - 1] == '\n')) buf[--L] = 0;
        char* w[16];
        int nw;
        om_split(buf, w, &nw, 16);
        if (nw == 0 || !strcmp(w[0], "%")) continue;
        if (!strcmp(w[0], "NDIME")) state = S_NDIME;
        else if (!strcmp(w[0], "NPOIN")) state = S_NPOIN;
        else if (!strcmp(w[0], "NELEM")) state = S_NELEM;
        else if (!strcmp(w[0], "NMARK")) state = S_NMARK;
        if (state == S_NDIME) {
            if (!(nw == 3 && !strcmp(w[2], "2"))) OM_FAIL("SU2 mesh dimension is not 2D");
        } else if (state == S_NPOIN && w[0][0] != 'N') {
            if (nw < 2) OM_FAIL("bad node line");
            if (nnode == capnode) {
                capnode *= 2;
                nx = (double*)realloc(nx, capnode * sizeof(double));
                ny = (double*)realloc(ny, capnode * sizeof(double));
                nid = (int*)realloc(nid, capnode * sizeof(int));
            }
            nx[nnode] = strtod(w[0], NULL);
            ny[nnode] = strtod(w[1], NULL);
            int id = -1;
            if (nw == 3) id = (int)strtod(w[2], NULL) + 1;
            else if (nw == 4) id = (int)strtod(w[3], NULL) + 1;
            nid[nnode] = id;
            if (id > maxnodeID) maxnodeID = id;
            nnode++;
        } else if (state == S_NELEM && w[0][0] != 'N') {
            int t[3][3];
            int nt = 0;
            if (!strcmp(w[0], "5")) {
                if (nw < 4) OM_FAIL("bad element line");
                t[0][0] = (int)strtod(w[1], NULL) + 1; t[0][1] = (int)strtod(w[2], NULL) + 1; t[0][2] = (int)strtod(w[3], NULL) + 1;
                nt = 1;
            } else if (!strcmp(w[0], "9")) {
                if (nw < 5) OM_FAIL("bad element line");
                int q1 = (int)strtod(w[1], NULL) + 1, q2 = (int)strtod(w[2], NULL) + 1;
                int q3 = (int)strtod(w[3], NULL) + 1, q4 = (int)strtod(w[4], NULL) + 1;
                /* quads always split: (n0,n1,n3) then (n3,n1,n2), SU2MeshReader.cpp:104-119 */
                t[0][0] = q1; t[0][1] = q2; t[0][2] = q4;
                t[1][0] = q4; t[1][1] = q2; t[1][2] = q3;
                nt = 2;
            }
            for (int k = 0; k < nt; k++) {
                if (ntri == captri) { captri *= 2; tri = (int*)realloc(tri, captri * 3 * sizeof(int)); }
                tri[3 * ntri] = t[k][0]; tri[3 * ntri + 1] = t[k][1]; tri[3 * ntri + 2] = t[k][2];
                ntri++;
            }
        } else if (state == S_NMARK) {
            if (!strcmp(w[0], "NMARK") || !strcmp(w[0], "MARKER_ELEMS")) {
            } else if (!strcmp(w[0], "MARKER_TAG")) {
                if (nw < 3) OM_FAIL("bad MARKER_TAG line");
                mk = (om_marker*)realloc(mk, (size_t)(nmk + 1) * sizeof(om_marker));
                memset(&mk[nmk], 0, sizeof(om_marker));
                strncpy(mk[nmk].name, w[2], 63);
                nmk++;
            } else {
                if (nmk == 0 || nw < 3) OM_FAIL("bad marker line");
                om_marker* c = &mk[nmk - 1];
                if (c->nedge == c->cap) {
                    c->cap = c->cap ? 2 * c->cap : 64;
                    c->e = (om_pair*)realloc(c->e, (size_t)c->cap * sizeof(om_pair));
                }
                c->e[c->nedge].n0 = atoi(w[1]) + 1;
                c->e[c->nedge].n1 = atoi(w[2]) + 1;
                c->nedge++;
            }
        }
    }
    fclose(f);
    f = NULL;
    if (nnode == 0 || ntri == 0) OM_FAIL("no nodes or elements");

    /* scaleMesh, SU2MeshReader.cpp:157-173 */
    {
        double res = scale - 1.0;
        if (!(res > -0.01 && res < 0.01)) {
            if (scale < 0.0) OM_FAIL("mesh scale factor should be positive");
            for (size_t i = 0; i < nnode; i++) { nx[i] *= scale; ny[i] *= scale; }
        }
    }
    /* pNodeTable: ID -> node index (FVM_2D.cpp:25-34); GPUID = vector index */
    idx = (int*)malloc((size_t)(maxnodeID + 1) * sizeof(int));
    for (int i = 0; i <= maxnodeID; i++) idx[i] = -1;
    for (size_t i = 0; i < nnode; i++) if (nid[i] >= 0) idx[nid[i]] = (int)i;

    const int N = (int)ntri;
    m = (om_mesh*)calloc(1, sizeof(om_mesh));
    m->N = N;
    m->V = (int)nnode;
    m->NB = nmk;
    m->elem_vol = (double*)malloc((size_t)N * sizeof(double));
    m->elem_xy = (double*)malloc((size_t)2 * N * sizeof(double));
    /* FVM_2D::iniEdges, FVM_2D.cpp:50-70: CCW fix by the signed area */
    for (int e = 0; e < N; e++) {
        int* t = &tri[3 * e];
        double xn[3], yn[3];
        for (int i = 0; i < 3; i++) {
            if (t[i] < 0 || t[i] > maxnodeID || idx[t[i]] < 0) OM_FAIL("element %d names an unknown node", e);
            xn[i] = nx[idx[t[i]]];
            yn[i] = ny[idx[t[i]]];
        }
        double area = 0.5 * (xn[0] * (yn[1] - yn[2]) + xn[1] * (yn[2] - yn[0]) + xn[2] * (yn[0] - yn[1]));
        if (area < 0) {
            m->elem_vol[e] = -area;
            int n1 = t[1]; t[1] = t[2]; t[2] = n1;
        } else {
            m->elem_vol[e] = area;
        }
    }
    /* edges in first-seen order; the first owner is L, the second R
     * (FVM_2D.cpp:72-81, iniEdges_registerSingle 116-134) */
    h.cap = 1;
    while (h.cap < (size_t)N * 4) h.cap <<= 1;
    h.key = (uint64_t*)malloc(h.cap * sizeof(uint64_t));
    h.val = (int*)malloc(h.cap * sizeof(int));
    for (size_t i = 0; i < h.cap; i++) h.val[i] = -1;
    size_t capE = (size_t)N * 2 + 16;
    en0 = (int*)malloc(capE * sizeof(int)); en1 = (int*)malloc(capE * sizeof(int));
    eL = (int*)malloc(capE * sizeof(int)); eR = (int*)malloc(capE * sizeof(int));
    int E = 0;
    pedges = (int*)malloc((size_t)3 * N * sizeof(int));
    for (int e = 0; e < N; e++) {
        const int* t = &tri[3 * e];
        for (int k = 0; k < 3; k++) {
            int a = t[k], b = t[(k + 1) % 3];
            int ei = om_emap_get(&h, a, b);
            if (ei < 0) {
                if ((size_t)E == capE) {
                    capE *= 2;
                    en0 = (int*)realloc(en0, capE * sizeof(int)); en1 = (int*)realloc(en1, capE * sizeof(int));
                    eL = (int*)realloc(eL, capE * sizeof(int)); eR = (int*)realloc(eR, capE * sizeof(int));
                }
                en0[E] = a; en1[E] = b; eL[E] = e; eR[E] = -1;
                om_emap_put(&h, a, b, E);
                E++;
            } else {
                eR[ei] = e;
            }
        }
    }
    /* pEdges[0..2] = edge(n0,n1), edge(n1,n2), edge(n2,n0); centroid = (sum of x)/3
     * (FVM_2D::iniElement_xy_pEdges, FVM_2D.cpp:165-185) */
    for (int e = 0; e < N; e++) {
        const int* t = &tri[3 * e];
        double sx = 0, sy = 0;
        for (int i = 0; i < 3; i++) { sx += nx[idx[t[i]]]; sy += ny[idx[t[i]]]; }
        m->elem_xy[e] = sx / 3.0;
        m->elem_xy[N + e] = sy / 3.0;
        for (int k = 0; k < 3; k++) pedges[3 * e + k] = om_emap_get(&h, t[k], t[(k + 1) % 3]);
    }
    m->E = E;
    m->edge_nodes = (int*)malloc((size_t)2 * E * sizeof(int));
    m->edge_L = (int*)malloc((size_t)E * sizeof(int));
    m->edge_R = (int*)malloc((size_t)E * sizeof(int));
    m->edge_set = (int*)malloc((size_t)E * sizeof(int));
    m->edge_pair = (int*)malloc((size_t)E * sizeof(int));
    m->edge_len = (double*)malloc((size_t)E * sizeof(double));
    m->edge_dist = (double*)malloc((size_t)E * sizeof(double));
    m->edge_xy = (double*)malloc((size_t)2 * E * sizeof(double));
    m->edge_normal = (double*)malloc((size_t)2 * E * sizeof(double));
    eset = m->edge_set;
    for (int i = 0; i < E; i++) eset[i] = -1;

    /* boundary sets (SU2MeshReader::process, SU2MeshReader.cpp:201-243) */
    m->bc_type = (int*)malloc((size_t)(nmk > 0 ? nmk : 1) * sizeof(int));
    int* pp_type = (int*)malloc((size_t)(nmk + 1) * sizeof(int));
    int* pp_s0 = (int*)malloc((size_t)(nmk + 1) * sizeof(int));
    int* pp_s1 = (int*)malloc((size_t)(nmk + 1) * sizeof(int));
    int npp = 0;
    int** setedges = (int**)calloc((size_t)(nmk > 0 ? nmk : 1), sizeof(int*));
    for (int s = 0; s < nmk; s++) {
        int bt = om_bc_type(mk[s].name, equation);
        if (bt == -2) { free(pp_type); free(pp_s0); free(pp_s1); for (int q = 0; q < s; q++) free(setedges[q]); free(setedges); OM_FAIL("unknown boundary type %s", mk[s].name); }
        m->bc_type[s] = bt;
        setedges[s] = (int*)malloc((size_t)(mk[s].nedge > 0 ? mk[s].nedge : 1) * sizeof(int));
        for (int k = 0; k < mk[s].nedge; k++) {
            int ei = om_emap_get(&h, mk[s].e[k].n0, mk[s].e[k].n1);
            if (ei < 0) { free(pp_type); free(pp_s0); free(pp_s1); for (int q = 0; q <= s; q++) free(setedges[q]); free(setedges); OM_FAIL("boundary edge not in mesh"); }
            eset[ei] = s + 1;
            setedges[s][k] = ei;
        }
        if (bt >= BC_PERIODIC_0 && bt <= BC_PERIODIC_9) {
            int ip = -1;
            for (int q = 0; q < npp; q++) if (pp_type[q] == bt) ip = q;
            if (ip != -1) pp_s1[ip] = s + 1;
            else { pp_type[npp] = bt; pp_s0[npp] = s + 1; pp_s1[npp] = -1; npp++; }
        }
    }
    /* edge lengths: computed in myfloat, rounded through float (FVM_2D.cpp:189-198, Edge_2D.cpp:19-28);
     * distance of cell centres in float arithmetic (Edge_2D.cpp:30-52) */
    for (int i = 0; i < E; i++) {
        int a = idx[en0[i]], b = idx[en1[i]];
        double x0 = nx[a], y0 = ny[a], x1 = nx[b], y1 = ny[b];
        m->edge_len[i] = (double)(float)sqrt((x0 - x1) * (x0 - x1) + (y0 - y1) * (y0 - y1));
        float xl = (float)m->elem_xy[eL[i]], yl = (float)m->elem_xy[N + eL[i]], xr, yr, dx, dy;
        if (eR[i] < 0) {
            xr = (float)((x0 + x1) / 2.0);
            yr = (float)((y0 + y1) / 2.0);
            dx = xr - xl; dy = yr - yl;
            m->edge_dist[i] = (double)(float)(2.0f * sqrtf(dx * dx + dy * dy));
        } else {
            xr = (float)m->elem_xy[eR[i]]; yr = (float)m->elem_xy[N + eR[i]];
            dx = xr - xl; dy = yr - yl;
            m->edge_dist[i] = (double)(float)sqrtf(dx * dx + dy * dy);
        }
    }
    /* BoundaryManager_2D::checkPeriodPairs, BoundaryManager_2D.cpp:183-255 */
    for (int q = 0; q < npp; q++) {
        if (pp_s0[q] == -1 || pp_s1[q] == -1) { free(pp_type); free(pp_s0); free(pp_s1); for (int s = 0; s < nmk; s++) free(setedges[s]); free(setedges); OM_FAIL("periodic boundaries do not appear in pairs"); }
        int s0 = pp_s0[q] - 1, s1 = pp_s1[q] - 1;
        int n = mk[s0].nedge;
        if (n != mk[s1].nedge) { free(pp_type); free(pp_s0); free(pp_s1); for (int s = 0; s < nmk; s++) free(setedges[s]); free(setedges); OM_FAIL("periodic edge counts do not match"); }
#define EX(ei) ((nx[idx[en0[ei]]] + nx[idx[en1[ei]]]) / 2.0)
#define EY(ei) ((ny[idx[en0[ei]]] + ny[idx[en1[ei]]]) / 2.0)
        double tx = EX(setedges[s1][n - 1]) - EX(setedges[s0][0]);
        double ty = EY(setedges[s1][n - 1]) - EY(setedges[s0][0]);
        for (int k = 0; k < n; k++) {
            double x1r = EX(setedges[s0][k]) + tx, y1r = EY(setedges[s0][k]) + ty;
            double x1 = EX(setedges[s1][n - 1 - k]), y1 = EY(setedges[s1][n - 1 - k]);
            double rx = x1 - x1r, ry = y1 - y1r;
            double rs = rx * rx + ry * ry, ts = tx * tx + ty * ty;
            if (rs / ts >= 0.0001) { free(pp_type); free(pp_s0); free(pp_s1); for (int s = 0; s < nmk; s++) free(setedges[s]); free(setedges); OM_FAIL("periodic boundary not translatable"); }
        }
#undef EX
#undef EY
    }

    /* OldDataConverter (FVMR/src/solvers/OldDataConverter.cpp:35-195) */
    m->node_xy = (double*)malloc((size_t)2 * m->V * sizeof(double));
    for (int i = 0; i < m->V; i++) { m->node_xy[i] = nx[i]; m->node_xy[m->V + i] = ny[i]; }
    m->elem_nodes = (int*)malloc((size_t)4 * N * sizeof(int));
    m->elem_edges = (int*)malloc((size_t)4 * N * sizeof(int));
    m->elem_nbrs = (int*)malloc((size_t)4 * N * sizeof(int));
    for (int e = 0; e < N; e++) {
        for (int j = 0; j < 3; j++) {
            m->elem_nodes[j * N + e] = idx[tri[3 * e + j]];
            m->elem_edges[j * N + e] = pedges[3 * e + j];
        }
        m->elem_nodes[3 * N + e] = -1;
        m->elem_edges[3 * N + e] = -1;
        for (int j = 0; j < 4; j++) m->elem_nbrs[j * N + e] = -1;
        /* Element_2D::findNeighbor, Element_2D.cpp:19-48 */
        for (int j = 0; j < 3; j++) {
            int ei = pedges[3 * e + j];
            int nb = -1;
            if (eL[ei] == e) nb = eR[ei];
            else if (eR[ei] == e) nb = eL[ei];
            m->elem_nbrs[j * N + e] = nb;
        }
    }
    for (int i = 0; i < E; i++) {
        int a = idx[en0[i]], b = idx[en1[i]];
        m->edge_nodes[i] = a;
        m->edge_nodes[E + i] = b;
        m->edge_L[i] = eL[i];
        m->edge_R[i] = eR[i];
        m->edge_pair[i] = -1;
        m->edge_xy[i] = (m->node_xy[a] + m->node_xy[b]) / 2.0;
        m->edge_xy[E + i] = (m->node_xy[m->V + a] + m->node_xy[m->V + b]) / 2.0;
        double dx = m->node_xy[b] - m->node_xy[a];
        double dy = m->node_xy[m->V + b] - m->node_xy[m->V + a];
        m->edge_normal[i] = dy / m->edge_len[i];
        m->edge_normal[E + i] = -dx / m->edge_len[i];
    }
    /* periodic partner: reversed index in the paired set (BoundaryManager_2D.cpp:304-323) */
    for (int s = 0; s < nmk; s++) {
        int bt = m->bc_type[s];
        if (!(bt >= BC_PERIODIC_0 && bt <= BC_PERIODIC_9)) continue;
        int other = -1;
        for (int q = 0; q < npp; q++)
            if (pp_type[q] == bt) { other = (pp_s0[q] == s + 1) ? pp_s1[q] : pp_s0[q]; break; }
        int n = mk[s].nedge;
        for (int k = 0; k < n; k++) {
            int ei = setedges[s][k];
            int index0 = k; /* getEdgeIndex returns the first position */
            for (int q = 0; q < k; q++) if (setedges[s][q] == ei) { index0 = q; break; }
            int pe = setedges[other - 1][n - 1 - index0];
            m->edge_R[ei] = m->edge_L[pe];
            m->edge_pair[ei] = pe;
        }
    }
    free(pp_type); free(pp_s0); free(pp_s1);
    for (int s = 0; s < nmk; s++) free(setedges[s]);
    free(setedges);
    free(nx); free(ny); free(nid); free(tri); free(idx); free(pedges);
    free(en0); free(en1); free(eL); free(eR);
    free(h.key); free(h.val);
    for (int s = 0; s < nmk; s++) free(mk[s].e);
    free(mk);
    return m;
fail:
    if (f) fclose(f);
    free(nx); free(ny); free(nid); free(tri); free(idx); free(pedges);
    free(en0); free(en1); free(eL); free(eR);
    free(h.key); free(h.val);
    for (int s = 0; s < nmk; s++) free(mk[s].e);
    free(mk);
    if (m) { m->edge_set = eset; om_mesh_free(m); }
    return NULL;
}

void om_mesh_free(om_mesh* m) {
    if (!m) return;
    free(m->node_xy); free(m->elem_nodes); free(m->elem_edges); free(m->elem_nbrs);
    free(m->elem_xy); free(m->elem_vol); free(m->edge_nodes); free(m->edge_L); free(m->edge_R);
    free(m->edge_set); free(m->edge_pair); free(m->edge_len); free(m->edge_dist); free(m->edge_xy);
    free(m->edge_normal); free(m->bc_type);
    free(m);
}

/* ------------------------------------------------------------------------ */
/* physics                                                                   */
/* ------------------------------------------------------------------------ */

/* U2ruvp_host / ruvp2U_host, FVMR/src/math/PhysicalKernel.h:11-27 */
static inline void U2ruvp(const double U[4], double r[4], double gamma) {
    r[0] = U[0];
    r[1] = U[1] / U[0];
    r[2] = U[2] / U[0];
    r[3] = r[0] * (gamma - 1) * (U[3] / U[0] - (r[1] * r[1] + r[2] * r[2]) * 0.5);
}
static inline void ruvp2U(const double r[4], double U[4], double gamma) {
    U[0] = r[0];
    U[1] = r[0] * r[1];
    U[2] = r[0] * r[2];
    U[3] = r[3] / (gamma - 1) + 0.5 * r[0] * (r[1] * r[1] + r[2] * r[2]);
}
/* Restrict::outOfRange, FVMR/src/space/restrict/Restrict.h:15-23 */
static inline int out_of_range(const double r[4]) {
    return r[0] < OM_RHO_MIN || r[0] > OM_RHO_MAX || r[3] < OM_P_MIN || r[3] > OM_P_MAX;
}

void om_ruvp_from_mach(double Ma, double AoA, double T0, double p0, double gamma, double R, double* ruvp) {
    /* AirParameterConverter::get_ruvp_by_Ma_AoA_T0_p0_gamma_R, FVMR/src/input/AirParameterConverter.cpp:3-24 */
    const double PI = 3.1415926535897;
    double T = T0 / (1.0 + (gamma - 1.0) / 2.0 * Ma * Ma);
    double p = p0 * pow(T / T0, gamma / (gamma - 1.0));
    double c = sqrt(gamma * R * T);
    ruvp[0] = p / (R * T);
    ruvp[1] = c * Ma * cos(AoA / 180 * PI);
    ruvp[2] = c * Ma * sin(AoA / 180 * PI);
    ruvp[3] = p;
}

int om_init_field(const om_mesh* m, const om_params* p, int ic, const double* vortex, double* U) {
    const int N = m->N;
    const double gamma = p->gamma;
    if (ic == 1) { /* FieldInitializer::setInitialUniform, FieldInitializer.cpp:129-137 */
        double u4[4];
        ruvp2U(p->inf, u4, gamma);
        for (int e = 0; e < N; e++) for (int j = 0; j < 4; j++) U[j * N + e] = u4[j];
        return 0;
    }
    if (ic == 2) { /* FieldInitializer::setInitialIsentropicVortex, FieldInitializer.cpp:139-177 */
        const double xc = vortex[0], yc = vortex[1], chi = vortex[2];
        const double chi2 = chi * chi, ga1 = gamma - 1.0;
        const double two_pi = 2.0 * OM_PI, pi2 = OM_PI * OM_PI;
        const double c_du = chi / two_pi;
        const double c_dT = ga1 * chi2 / (8. * gamma * pi2);
        for (int e = 0; e < N; e++) {
            double dx = m->elem_xy[e] - xc, dy = m->elem_xy[N + e] - yc;
            double r2 = dx * dx + dy * dy;
            double one_minus_r2 = 1.0 - r2;
            double c_distance = exp(0.5 * one_minus_r2);
            double du = c_du * c_distance * (-dy);
            double dv = c_du * c_distance * dx;
            double u = p->inf[1] + du, v = p->inf[2] + dv;
            double dT = -c_dT * exp(one_minus_r2);
            double rho = pow(p->inf[3] + dT, 1. / ga1);
            double pr = rho * (p->inf[3] + dT);
            double r[4] = {rho, u, v, pr}, u4[4];
            ruvp2U(r, u4, gamma);
            for (int j = 0; j < 4; j++) U[j * N + e] = u4[j];
        }
        return 0;
    }
    if (ic == 3) { /* FieldInitializer::setInitialShockTube, FieldInitializer.cpp:179-222 */
        double sx = p->shock[0], sy = p->shock[1], snx = p->shock[2], sny = p->shock[3];
        if (snx == 0.0 && sny == 0.0) snx = 1.0;
        double length_inv = 1.0 / sqrt(snx * snx + sny * sny);
        snx *= length_inv;
        sny *= length_inv;
        double ui[4], uo[4];
        ruvp2U(p->inlet, ui, gamma);
        ruvp2U(p->outlet, uo, gamma);
        for (int e = 0; e < N; e++) {
            double x = m->elem_xy[e], y = m->elem_xy[N + e];
            int inlet;
            if (snx == 1.0) inlet = x < sx;
            else inlet = !((x - sx) * snx + (y - sy) * sny > 0);
            for (int j = 0; j < 4; j++) U[j * N + e] = inlet ? ui[j] : uo[j];
        }
        return 0;
    }
    if (ic == 4) { /* FieldInitializer::setInitialDoubleShockReflection, FieldInitializer.cpp:224-260,
                      with isUpStreamOfShock_forElement, CBoundaryDoubleShockReflect.cpp:17-33 */
        double angle_rad = p->dsr[2] * OM_PI / 180.0;
        double norm_x = -sin(angle_rad), norm_y = cos(angle_rad);
        double ui[4], uo[4];
        ruvp2U(p->inlet, ui, gamma);
        ruvp2U(p->outlet, uo, gamma);
        for (int e = 0; e < N; e++) {
            double r_x = m->elem_xy[e] - p->dsr[0], r_y = m->elem_xy[N + e] - p->dsr[1];
            int up = r_x * norm_x + r_y * norm_y > 0;
            for (int j = 0; j < 4; j++) U[j * N + e] = up ? ui[j] : uo[j];
        }
        return 0;
    }
    return -1;
}

/* ---- gradients ---------------------------------------------------------- */

/* GradientLeastSquare_2, FVMR/src/space/gradient/Gradient.cpp:160-246, with the
 * matrix helpers of FVMR/src/math/MatrixKernel.h:21-93 */
static int grad_lsq(const om_mesh* m, const om_params* p, const double* U, double* gx, double* gy) {
    const int N = m->N;
    int bad = 0;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < N; e++) {
        int nb[3], nvn = 0;
        for (int j = 0; j < 3; j++) if (m->elem_nbrs[j * N + e] != -1) nb[nvn++] = m->elem_nbrs[j * N + e];
        if (nvn <= 0) {
#pragma omp critical
            bad = 1;
            continue;
        }
        double dX[6], dU[12], dXt[6], A[4], B[6], G[8];
        for (int k = 0; k < nvn; k++) {
            dX[k * 2 + 0] = m->elem_xy[nb[k]] - m->elem_xy[e];
            dX[k * 2 + 1] = m->elem_xy[N + nb[k]] - m->elem_xy[N + e];
            for (int v = 0; v < 4; v++) dU[k * 4 + v] = U[v * N + nb[k]] - U[v * N + e];
        }
        for (int x = 0; x < nvn; x++) for (int y = 0; y < 2; y++) dXt[y * nvn + x] = dX[x * 2 + y];
        for (int x = 0; x < 2; x++) for (int y = 0; y < 2; y++) {
            A[x * 2 + y] = 0.0;
            for (int z = 0; z < nvn; z++) A[x * 2 + y] += dXt[x * nvn + z] * dX[z * 2 + y];
        }
        { /* inv_2x2 (MatrixKernel.h:45-59): the reference turns every det >= EPS into -EPS */
            double det = A[0] * A[3] - A[1] * A[2];
            if (p->lsq_det_ref) {
                if (det >= 0 && det < OM_EPS) det = OM_EPS;
                else if (det > -OM_EPS) det = -OM_EPS;
            } else {
                if (det >= 0 && det < OM_EPS) det = OM_EPS;
                else if (det < 0 && det > -OM_EPS) det = -OM_EPS;
            }
            double inv_det = 1.0 / det;
            double ia = A[3] * inv_det, ib = -A[1] * inv_det, ic = -A[2] * inv_det, id = A[0] * inv_det;
            A[0] = ia; A[1] = ib; A[2] = ic; A[3] = id;
        }
        for (int x = 0; x < 2; x++) for (int y = 0; y < nvn; y++) {
            B[x * nvn + y] = 0.0;
            for (int z = 0; z < 2; z++) B[x * nvn + y] += A[x * 2 + z] * dXt[z * nvn + y];
        }
        for (int x = 0; x < 2; x++) for (int y = 0; y < 4; y++) {
            G[x * 4 + y] = 0.0;
            for (int z = 0; z < nvn; z++) G[x * 4 + y] += B[x * nvn + z] * dU[z * 4 + y];
        }
        for (int v = 0; v < 4; v++) { gx[v * N + e] = G[v]; gy[v * N + e] = G[4 + v]; }
    }
    return bad ? -3 : 0;
}

/* GradientGreenGauss_2, FVMR/src/space/gradient/Gradient.cpp:248-458 */
static void grad_gg(const om_mesh* m, const double* U, double* gx, double* gy) {
    const int N = m->N, E = m->E;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < N; c++) {
        double volC = m->elem_vol[c];
        int eid[4], etype[4], sign[4], out[4];
        double Sx[4] = {0}, Sy[4] = {0}, gC[4] = {0};
        for (int i = 0; i < 4; i++) {
            eid[i] = m->elem_edges[i * N + c];
            if (!(eid[i] >= 0 && eid[i] < E)) eid[i] = -1;
            etype[i] = -1; sign[i] = 0; out[i] = -1;
        }
        for (int i = 0; i < 4; i++) if (eid[i] != -1) etype[i] = m->edge_set[eid[i]];
        for (int i = 0; i < 4; i++) {
            int ei = eid[i];
            if (ei == -1) continue;
            if (c != m->edge_R[ei]) { sign[i] = 1; out[i] = m->edge_R[ei]; }
            else { sign[i] = -1; out[i] = m->edge_L[ei]; }
        }
        for (int i = 0; i < 4; i++) {
            int ei = eid[i];
            if (ei == -1) continue;
            double nxx = m->edge_normal[ei], nyy = m->edge_normal[E + ei], len = m->edge_len[ei];
            Sx[i] = nxx * len;
            Sy[i] = nyy * len;
        }
        for (int i = 0; i < 4; i++) {
            int ei = eid[i];
            if (ei == -1) continue;
            int o = out[i];
            if (o != -1) {
                double fx = m->edge_xy[ei], fy = m->edge_xy[E + ei];
                double Cx = m->elem_xy[c], Cy = m->elem_xy[N + c];
                double Fx = m->elem_xy[o], Fy = m->elem_xy[N + o];
                if (etype[i] != -1) { /* periodic: shift F by the face-pair offset */
                    int pe = m->edge_pair[ei];
                    double shx = fx - m->edge_xy[pe], shy = fy - m->edge_xy[E + pe];
                    Fx += shx;
                    Fy += shy;
                }
                double dFf = m_dist2(Fx, Fy, fx, fy);
                double dFC = m_dist2(Fx, Fy, Cx, Cy);
                if (dFC < OM_EPS) dFC = OM_EPS;
                gC[i] = dFf / dFC;
            } else {
                gC[i] = 0.5;
            }
        }
        for (int v = 0; v < 4; v++) {
            double s0 = 0, s1 = 0;
            for (int i = 0; i < 4; i++) {
                if (eid[i] == -1) continue;
                double phiC = U[v * N + c], phif;
                if (out[i] != -1) {
                    double phiF = U[v * N + out[i]];
                    double g = gC[i], g1 = 1.0 - g;
                    phif = g * phiC + g1 * phiF;
                } else {
                    phif = phiC;
                }
                s0 += phif * Sx[i] * sign[i];
                s1 += phif * Sy[i] * sign[i];
            }
            gx[v * N + c] = 1 / volC * s0;
            gy[v * N + c] = 1 / volC * s1;
        }
    }
}

/* LimiterBarth, FVMR/src/space/gradient/Gradient.cpp:58-114 */
static void limiter_barth(const om_mesh* m, const double* U, double* gx, double* gy) {
    const int N = m->N, V = m->V;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < N; e++) {
        int nb[3], nvn = 0;
        for (int j = 0; j < 3; j++) if (m->elem_nbrs[j * N + e] != -1) nb[nvn++] = m->elem_nbrs[j * N + e];
        for (int v = 0; v < 4; v++) {
            double Uc = U[v * N + e], lo = Uc, hi = Uc;
            for (int j = 0; j < nvn; j++) {
                lo = m_min(lo, U[v * N + nb[j]]);
                hi = m_max(hi, U[v * N + nb[j]]);
            }
            double phi = 1.0;
            for (int j = 0; j < 3; j++) {
                int nd = m->elem_nodes[j * N + e];
                double xn = m->node_xy[nd], yn = m->node_xy[V + nd];
                double Un = U[v * N + e] + gx[v * N + e] * (xn - m->elem_xy[e]) + gy[v * N + e] * (yn - m->elem_xy[N + e]);
                double dn = Un - Uc, dhi = hi - Uc, dlo = lo - Uc, phin = 1.0;
                if (dn > 0) { dn += OM_EPS; phin = m_min(1, dhi / dn); }
                else if (dn < 0) { dn -= OM_EPS; phin = m_min(1, dlo / dn); }
                phi = m_min(phi, phin);
            }
            gx[v * N + e] *= phi;
            gy[v * N + e] *= phi;
        }
    }
}

/* ---- edge fluxes --------------------------------------------------------- */

/* get_Uvector_reconstruct_2, FVMR/src/space/Flux.cpp:28-55 */
static inline void reconstruct(const om_mesh* m, const om_params* p, const double* U, const double* gx, const double* gy,
                               double x, double y, int c, double out[4]) {
    const int N = m->N;
    for (int v = 0; v < 4; v++) {
        if (p->reconstruct == 3002)
            out[v] = U[v * N + c] + gx[v * N + c] * (x - m->elem_xy[c]) + gy[v * N + c] * (y - m->elem_xy[N + c]);
        else
            out[v] = U[v * N + c];
    }
    double r[4];
    U2ruvp(out, r, p->gamma);
    if (out_of_range(r)) for (int v = 0; v < 4; v++) out[v] = U[v * N + c];
}

/* get_UR_wallNonViscous, Flux.cpp:57-71 */
static inline void ghost_slip(const double UL[4], double UR[4], double nx, double ny) {
    double uxL = UL[1] / UL[0], uyL = UL[2] / UL[0];
    double unL = uxL * nx + uyL * ny;
    double utL = uxL * ny - uyL * nx;
    double unR = -unL, utR = utL;
    double uxR = unR * nx + utR * ny;
    double uyR = unR * ny - utR * nx;
    UR[0] = UL[0];
    UR[1] = UR[0] * uxR;
    UR[2] = UR[0] * uyR;
    UR[3] = UL[3];
}

/* get_UR_farField, Flux.cpp:81-163 */
static inline int ghost_farfield(const double UL[4], const double* inf, double UR[4], double nx, double ny, double gamma) {
    double ga1 = gamma - 1;
    double rho_f = inf[0], u_f = inf[1], v_f = inf[2], p_f = inf[3];
    double re4[4];
    U2ruvp(UL, re4, gamma);
    double rho_e = re4[0], u_e = re4[1], v_e = re4[2], p_e = re4[3];
    double a2_f = gamma * p_f / rho_f;
    double af = sqrt(a2_f);
    double ae = sqrt(gamma * p_e / rho_e);
    double qnf = u_f * nx + v_f * ny;
    double qne = u_e * nx + v_e * ny;
    double rf = qnf - 2.0 * af / ga1;
    double re = qne + 2.0 * ae / ga1;
    double qn = 0.5 * (re + rf);
    double as = ga1 * (re - rf) / 4.0;
    double rho0 = 1, u0 = 0, v0 = 0, p0 = 1;
    if (qn <= -as) {
        rho0 = rho_f; u0 = u_f; v0 = v_f; p0 = p_f;
    } else if (qn < 0) {
        double son = p_f / pow(rho_f, gamma);
        double qtx = u_f - qnf * nx, qty = v_f - qnf * ny;
        rho0 = pow((as * as / son / gamma), 1.0 / ga1);
        u0 = qtx + qn * nx;
        v0 = qty + qn * ny;
        p0 = as * as * rho0 / gamma;
    } else if (qn < as) {
        double son = p_e / pow(rho_e, gamma);
        double qtx = u_e - qne * nx, qty = v_e - qne * ny;
        rho0 = pow((as * as / son / gamma), 1.0 / ga1);
        u0 = qtx + qn * nx;
        v0 = qty + qn * ny;
        p0 = as * as * rho0 / gamma;
    } else {
        rho0 = rho_e; u0 = u_e; v0 = v_e; p0 = p_e;
    }
    double r0[4] = {rho0, u0, v0, p0};
    if (out_of_range(r0)) return -4;
    ruvp2U(r0, UR, gamma);
    return 0;
}

/* ConvectRoeCommon2d + RoeDissapationTerm2d, FVMR/src/space/convection/Roe.cpp:380-538 */
static inline void roe(const double UL[4], const double UR[4], double nx, double ny, double area, double F[4], double gamma) {
    double rl4[4], rr4[4];
    U2ruvp(UL, rl4, gamma);
    U2ruvp(UR, rr4, gamma);
    double rL = rl4[0], uL = rl4[1], vL = rl4[2], pL = rl4[3];
    double rR = rr4[0], uR = rr4[1], vR = rr4[2], pR = rr4[3];
    double ulnormaln = (nx * uL + ny * vL + 0.0);
    double urnormaln = (nx * uR + ny * vR + 0.0);
    double rulnormaln = rL * ulnormaln, rurnormaln = rR * urnormaln;
    double V2L = uL * uL + vL * vL, V2R = uR * uR + vR * vR;
    double ga1 = gamma - 1.0;
    double HL = pL * gamma / (rL * ga1) + 0.5 * V2L;
    double HR = pR * gamma / (rR * ga1) + 0.5 * V2R;
    F[0] = 0.5 * (rulnormaln + rurnormaln) * area;
    F[1] = 0.5 * (rulnormaln * uL + rurnormaln * uR + nx * (pL + pR)) * area;
    F[2] = 0.5 * (rulnormaln * vL + rurnormaln * vR + ny * (pL + pR)) * area;
    F[3] = 0.5 * (rulnormaln * HL + rurnormaln * HR - 0.0 * (pL + pR)) * area;
    /* dissipation (entropy fix disabled in the reference) */
    double rrorl = sqrt(rR / rL);
    double rrorlp1 = rrorl + 1.0;
    double rm = sqrt(rR * rL);
    double um = (uL + uR * rrorl) / rrorlp1;
    double vm = (vL + vR * rrorl) / rrorlp1;
    double Hm = (HL + HR * rrorl) / rrorlp1;
    double Vm2 = um * um + vm * vm;
    double am2 = ga1 * (Hm - 0.5 * Vm2);
    double am = sqrt(am2);
    double unormaln = um * nx + vm * ny;
    double eig1 = fabs(unormaln);
    double eig2 = fabs(unormaln + am);
    double eig3 = fabs(unormaln - am);
    double ER = HR - pR / rR, EL = HL - pL / rL;
    double Etm = Hm / gamma + ga1 / gamma * 0.5 * Vm2;
    double dW0 = rR - rL;
    double dW1 = rm * (uR - uL) + dW0 * um;
    double dW2 = rm * (vR - vL) + dW0 * vm;
    double dW3 = rm * (ER - EL) + dW0 * Etm;
    double astar = (eig2 + eig3) / 2.0;
    double Mstar = (eig2 - eig3) / 2.0 / am;
    double dunormaln = (nx * (uR - uL) + ny * (vR - vL));
    double dUroe = Mstar * dunormaln + (astar - eig1) * (pR - pL) / rm / am2;
    double dProe = Mstar * (pR - pL) + (astar - eig1) * rm * dunormaln;
    double d0 = 0.5 * (eig1 * dW0 + dUroe * rm) * area;
    double d1 = 0.5 * (eig1 * dW1 + dUroe * rm * um + dProe * nx) * area;
    double d2 = 0.5 * (eig1 * dW2 + dUroe * rm * vm + dProe * ny) * area;
    double d3 = 0.5 * (eig1 * dW3 + dUroe * rm * Hm + dProe * (unormaln - 0.0)) * area;
    F[0] -= 1.0 * d0;
    F[1] -= 1.0 * d1;
    F[2] -= 1.0 * d2;
    F[3] -= 1.0 * d3;
}

/* LocalLaxFriedrichs, FVMR/src/space/convection/LocalLaxFriedrichs.cpp:4-47 */
static inline void llf(const double UL[4], const double UR[4], double nx, double ny, double length, double F[4], double gamma) {
    double rl4[4], rr4[4];
    U2ruvp(UL, rl4, gamma);
    U2ruvp(UR, rr4, gamma);
    double rL = rl4[0], uL = rl4[1], vL = rl4[2], pL = rl4[3];
    double rR = rr4[0], uR = rr4[1], vR = rr4[2], pR = rr4[3];
    double unL = nx * uL + ny * vL, unR = nx * uR + ny * vR;
    double FnL[4], FnR[4];
    FnL[0] = rL * unL;
    FnL[1] = rL * unL * uL + nx * pL;
    FnL[2] = rL * unL * vL + ny * pL;
    double hl = pL * gamma / (rL * (gamma - 1.)) + 0.5 * (uL * uL + vL * vL);
    FnL[3] = rL * unL * hl;
    FnR[0] = rR * unR;
    FnR[1] = rR * unR * uR + nx * pR;
    FnR[2] = rR * unR * vR + ny * pR;
    double hr = pR * gamma / (rR * (gamma - 1.)) + 0.5 * (uR * uR + vR * vR);
    FnR[3] = rR * unR * hr;
    double lambdaMax = m_max(m_abs(unL) + sqrt(gamma * pL / rL), m_abs(unR) + sqrt(gamma * pR / rR));
    for (int i = 0; i < 4; i++) {
        F[i] = 0.5 * (FnL[i] + FnR[i] - lambdaMax * (UR[i] - UL[i]));
        F[i] *= length;
    }
}

/* edge_convection_flux_kernel, Flux.cpp:230-303 */
static int edge_flux(const om_mesh* m, const om_params* p, const double* U, const double* gx, const double* gy, int ei, double F[4]) {
    const int E = m->E;
    int setID = m->edge_set[ei], bType = -1;
    if (setID != -1) bType = m->bc_type[setID - 1];
    double nx = m->edge_normal[ei], ny = m->edge_normal[E + ei];
    double x = m->edge_xy[ei], y = m->edge_xy[E + ei];
    double length = m->edge_len[ei];
    int L = m->edge_L[ei], R = m->edge_R[ei];
    double UL[4] = {0}, UR[4] = {0};
    reconstruct(m, p, U, gx, gy, x, y, L, UL);
    switch (bType) {
    case BC_SYMMETRY:
    case BC_WALL_NONVISCOUS:
        ghost_slip(UL, UR, nx, ny);
        break;
    case BC_WALL_ADIABAT:
        if (p->wall_bc_ref) { /* Flux.cpp:73-79: U_R[1..2] negate a zero-initialised array */
            UR[0] = UL[0]; UR[1] = -UR[1]; UR[2] = -UR[2]; UR[3] = UL[3];
        } else {
            UR[0] = UL[0]; UR[1] = -UL[1]; UR[2] = -UL[2]; UR[3] = UL[3];
        }
        break;
    case BC_INLET:
        if (ghost_farfield(UL, p->inlet, UR, nx, ny, p->gamma)) return -4;
        break;
    case BC_OUTLET:
        if (ghost_farfield(UL, p->outlet, UR, nx, ny, p->gamma)) return -4;
        break;
    case BC_INF:
        if (ghost_farfield(UL, p->inf, UR, nx, ny, p->gamma)) return -4;
        break;
    case BC_DSR: { /* Flux.cpp:280-287 with isUpStreamOfShock_atBoundary_static_inline (Flux.cpp:21-26):
                      shock speed 20 (CBoundaryDoubleShockReflect.h:15), sqrt3 = sqrt(3.0) */
        double right = p->dsr[0] + (y + 20.0 * p->dsr_time) / sqrt(3.0);
        const double* far = (x < right) ? p->inlet : p->outlet;
        if (ghost_farfield(UL, far, UR, nx, ny, p->gamma)) return -4;
        break;
    }
    default:
        if (R != -1) {
            if (setID != -1) { /* periodic: reconstruct R at the partner edge's midpoint */
                int pe = m->edge_pair[ei];
                if (pe < 0 || pe >= E) return -6;
                reconstruct(m, p, U, gx, gy, m->edge_xy[pe], m->edge_xy[E + pe], R, UR);
            } else {
                reconstruct(m, p, U, gx, gy, x, y, R, UR);
            }
        }
    }
    if (p->flux_scheme == 2001) llf(UL, UR, nx, ny, length, F, p->gamma);
    else roe(UL, UR, nx, ny, length, F, p->gamma);
    return 0;
}

/* viscous_flux_kernel + helpers, FVMR/src/space/viscous_flux/ViscousFlux.cpp:63-168 and
 * ViscousFluxGPU.cu:7-124; Sutherland, ViscousFluxGPU.h:26-32 */
static inline void viscous_flux(const om_mesh* m, const om_params* p, const double* U, const double* gx, const double* gy,
                                int ei, double C1, double F[4]) {
    const int N = m->N, E = m->E;
    const int L = m->edge_L[ei], R = m->edge_R[ei];
    const double gamma = p->gamma, ga1 = gamma - 1.0;
    const double Cv = p->R / ga1, Cp = Cv * gamma;
    const double Pr = 0.72;
    double g[8], s[4];
    int hasR = !(R < 0 || R >= N);
    for (int v = 0; v < 4; v++) {
        double a = gx[v * N + L], b = gy[v * N + L];
        if (hasR) { a = 0.5 * (a + gx[v * N + R]); b = 0.5 * (b + gy[v * N + R]); }
        g[v] = a; g[4 + v] = b;
        double u = U[v * N + L];
        if (hasR) u = 0.5 * (u + U[v * N + R]);
        s[v] = u;
    }
    double rho = s[0], rhou = s[1], rhov = s[2], rhoE = s[3];
    double one_on_rho = 1.0 / rho;
    double u = rhou * one_on_rho, v = rhov * one_on_rho, Es = rhoE * one_on_rho;
    double dudx = one_on_rho * (g[1] - u * g[0]);
    double dvdx = one_on_rho * (g[2] - v * g[0]);
    double dudy = one_on_rho * (g[5] - u * g[4]);
    double dvdy = one_on_rho * (g[6] - v * g[4]);
    double dEdx = one_on_rho * (g[3] - Es * g[0]);
    double dEdy = one_on_rho * (g[7] - Es * g[4]);
    double one_on_Cv = 1.0 / Cv;
    double V2 = u * u + v * v;
    double T = one_on_Cv * (Es - 0.5 * V2);
    double dTdx = (dEdx - u * dudx - v * dvdx) * one_on_Cv;
    double dTdy = (dEdy - u * dudy - v * dvdy) * one_on_Cv;
    double mu = C1 * pow(T, 1.5) / (T + 110.4);
    const double NMD = -2.0 / 3.0;
    double div = dudx + dvdy;
    double txx = mu * (NMD * div + 2.0 * dudx);
    double tyy = mu * (NMD * div + 2.0 * dvdy);
    double txy = mu * (dudy + dvdx);
    /* the reference adds zero turbulent stresses (use_turbulence = false) */
    txx = txx + 0.0; tyy = tyy + 0.0; txy = txy + 0.0;
    double akmu = Cp * (mu / Pr);
    double Phix = akmu * dTdx + u * txx + v * txy;
    double Phiy = akmu * dTdy + u * txy + v * tyy;
    double nx = m->edge_normal[ei], ny = m->edge_normal[E + ei], area = m->edge_len[ei];
    F[0] -= 0.0;
    F[1] -= (txx * nx + txy * ny) * area;
    F[2] -= (txy * nx + tyy * ny) * area;
    F[3] -= (Phix * nx + Phiy * ny) * area;
}

static double sutherland_C1(const om_params* p) {
    return p->mu0 / pow(p->T0, 1.5) * (p->T0 + 110.4);
}

int om_rhs(const om_mesh* m, const om_params* p, const double* U, double* rhs, double* gx_out, double* gy_out) {
    const int N = m->N, E = m->E;
    double* gx = gx_out ? gx_out : (double*)malloc((size_t)4 * N * sizeof(double));
    double* gy = gy_out ? gy_out : (double*)malloc((size_t)4 * N * sizeof(double));
    double* ef = (double*)malloc((size_t)4 * E * sizeof(double));
    int rc = 0;
    /* Gradient dispatch, Gradient.cpp:116-158 */
    if (p->gradient == 1) rc = grad_lsq(m, p, U, gx, gy);
    else if (p->gradient == 2) grad_gg(m, U, gx, gy);
    else rc = -2;
    if (rc) goto done;
    if (p->limiter == 1) limiter_barth(m, U, gx, gy);
    else if (p->limiter != 0) { rc = -2; goto done; }
    /* calculateFluxHost, Flux.cpp:394-412 */
    {
        double C1 = sutherland_C1(p);
        int erc = 0;
#pragma omp parallel for schedule(static)
        for (int ei = 0; ei < E; ei++) {
            double F[4];
            int r = edge_flux(m, p, U, gx, gy, ei, F);
            if (r) {
#pragma omp critical
                erc = r;
                continue;
            }
            if (p->equation == 2) viscous_flux(m, p, U, gx, gy, ei, C1, F);
            for (int v = 0; v < 4; v++) ef[v * E + ei] = F[v];
        }
        rc = erc;
        if (rc) goto done;
    }
    /* add_edge_flux_to_element_flux, Flux.cpp:346-392, then the -1/vol scaling of
     * calculateFunctionF, FVMR/src/time/Evolve.cpp:106-111 */
#pragma omp parallel for schedule(static)
    for (int c = 0; c < N; c++) {
        double acc[4] = {0, 0, 0, 0};
        for (int i = 0; i < 4; i++) {
            int ei = m->elem_edges[i * N + c];
            if (!(ei >= 0 && ei < E)) continue;
            int sgn = (c != m->edge_R[ei]) ? 1 : -1;
            for (int v = 0; v < 4; v++) acc[v] += sgn * ef[v * E + ei];
        }
        double minus_one_on_volume = -1.0 / m->elem_vol[c];
        for (int v = 0; v < 4; v++) rhs[v * N + c] = minus_one_on_volume * acc[v];
    }
done:
    free(ef);
    if (!gx_out) free(gx);
    if (!gy_out) free(gy);
    return rc;
}

/* update_alphaC_host + get_minimus_dt_by_alphaC, FVMR/src/time/CalculateDt.cpp:10-85;
 * primitive variables as update_host_ruvp_Uold, CIteration.cpp:163-180 */
int om_dt(const om_mesh* m, const om_params* p, const double* U, double* dt_out, double* alpha_out) {
    const int N = m->N, E = m->E;
    const double gamma = p->gamma;
    double* rv = (double*)malloc((size_t)4 * N * sizeof(double));
    double* aC = alpha_out ? alpha_out : (double*)malloc((size_t)N * sizeof(double));
    int rc = 0;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        rv[i] = U[i];
        rv[N + i] = U[N + i] / U[i];
        rv[2 * N + i] = U[2 * N + i] / U[i];
        rv[3 * N + i] = rv[i] * (gamma - 1) * (U[3 * N + i] / U[i] - (rv[N + i] * rv[N + i] + rv[2 * N + i] * rv[2 * N + i]) * 0.5);
    }
    const double value_1 = m_max(4.0 / 3.0, gamma / p->Pr);
    const double C1 = sutherland_C1(p);
    for (int i = 0; i < N; i++) aC[i] = 0.0;
    for (int i = 0; i < E; i++) {
        int L = m->edge_L[i], R = m->edge_R[i];
        double rho, u, v, pr;
        if (R != -1) {
            rho = 0.5 * (rv[L] + rv[R]);
            u = 0.5 * (rv[N + L] + rv[N + R]);
            v = 0.5 * (rv[2 * N + L] + rv[2 * N + R]);
            pr = 0.5 * (rv[3 * N + L] + rv[3 * N + R]);
        } else {
            rho = rv[L]; u = rv[N + L]; v = rv[2 * N + L]; pr = rv[3 * N + L];
        }
        if (rho < 0 || pr < 0) { rc = -7; goto done; }
        double dx = m->edge_normal[i] * m->edge_len[i];
        double dy = m->edge_normal[E + i] * m->edge_len[i];
        const double length = m->edge_len[i];
        double unormal = u * dx + v * dy;
        double alpha = fabs(unormal) + sqrt(gamma * pr / rho) * sqrt(length);
        aC[L] += alpha;
        if (R != -1) aC[R] += alpha;
        if (p->equation == 2) {
            double temperature = pr / p->R / rho;
            double mu = C1 * pow(temperature, 1.5) / (temperature + 110.4);
            double alphaVis = 2.0 * length * value_1 * mu / rho;
            aC[L] += alphaVis / m->elem_vol[L];
            if (R != -1) aC[R] += alphaVis / m->elem_vol[R];
        }
    }
    {
        double dt = 1e10;
        for (int i = 0; i < N; i++) dt = m_min(dt, p->CFL * m->elem_vol[i] / aC[i]);
        *dt_out = dt;
    }
done:
    free(rv);
    if (!alpha_out) free(aC);
    return rc;
}

/* modifyElementFieldU2d(_kernel), FVMR/src/space/restrict/Restrict.cpp:7-90: cells in index
 * order, in place, replaced by the volume-weighted neighbour mean */
int om_restrict(const om_mesh* m, const om_params* p, double* U) {
    const int N = m->N;
    int count = 0;
    for (int e = 0; e < N; e++) {
        double u4[4], r[4];
        for (int v = 0; v < 4; v++) u4[v] = U[v * N + e];
        U2ruvp(u4, r, p->gamma);
        for (int v = 0; v < 4; v++) if (isnan(r[v])) return -1;
        if (!out_of_range(r)) continue;
        int nvn = 0;
        double Us[4] = {0, 0, 0, 0}, vs = 0.0;
        for (int i = 0; i < 4; i++) {
            int nb = m->elem_nbrs[i * N + e];
            if (nb == -1) continue;
            nvn++;
            if (p->restrict_ref) {
                for (int v = 0; v < 4; v++) { double vol = m->elem_vol[nb]; Us[v] += U[v * N + nb] * vol; vs += vol; }
            } else {
                double vol = m->elem_vol[nb];
                for (int v = 0; v < 4; v++) Us[v] += U[v * N + nb] * vol;
                vs += vol;
            }
        }
        if (nvn == 0) return -8;
        for (int v = 0; v < 4; v++) U[v * N + e] = Us[v] / vs;
        count++;
    }
    return count;
}

int om_run(const om_mesh* m, const om_params* p, double* U, int nsteps, double* t, double* dts, double* last_rhs) {
    const int N = m->N;
    const size_t M = (size_t)4 * N;
    double *U0 = (double*)malloc(M * sizeof(double)), *k1 = (double*)malloc(M * sizeof(double));
    double *k2 = (double*)malloc(M * sizeof(double)), *k3 = (double*)malloc(M * sizeof(double));
    double *Us = (double*)malloc(M * sizeof(double)), *U1 = (double*)malloc(M * sizeof(double));
    int rc = 0;
    om_params ps = *p; /* ps.dsr_time: the stage's clock, CIteration.cpp:60-62 and Evolve.cpp:43-77 */
    if (p->steady) {
        /* iteration_host's steady branch (CIteration.cpp:42-52): get_local_dt_host
         * (CalculateDt.cpp:66-72, 182-186), t += alphaC[0], evolve_explicit_localtimestep
         * (Evolve.cpp:115-125), then the positivity pass (CIteration.cpp:79).  The double-
         * Mach-reflection clock is not moved by this branch: it stays at p->dsr_time. */
        double* aC = (double*)malloc((size_t)N * sizeof(double));
        for (int s = 0; s < nsteps && rc == 0; s++) {
            double dmin;
            if ((rc = om_dt(m, p, U, &dmin, aC))) break;
            for (int i = 0; i < N; i++) aC[i] = p->CFL * m->elem_vol[i] / aC[i];
            *t += aC[0];
            if (dts) dts[s] = aC[0];
            if ((rc = om_rhs(m, p, U, k1, NULL, NULL))) break;
            #pragma omp parallel for schedule(static)
            for (int i = 0; i < N; i++)
                for (int j = 0; j < 4; j++) U[(size_t)j * N + i] += aC[i] * k1[(size_t)j * N + i];
            int r = om_restrict(m, p, U);
            if (r < 0) rc = r == -1 ? -9 : r;
        }
        free(aC);
        if (last_rhs && rc == 0) memcpy(last_rhs, k1, M * sizeof(double));
        free(U0); free(k1); free(k2); free(k3); free(Us); free(U1);
        return rc;
    }
    for (int s = 0; s < nsteps; s++) {
        double dt;
        rc = om_dt(m, p, U, &dt, NULL);
        if (rc) break;
        if (*t + dt > p->T_end) dt = p->T_end - *t; /* CIteration.cpp:59 */
        const double t0 = *t;
        *t += dt;
        if (dts) dts[s] = dt;
        memcpy(U0, U, M * sizeof(double));
        if (p->time_advance == 3101) { /* evolve_explicit_globaltimestep, Evolve.cpp:12-23 */
            ps.dsr_time = t0 + 0.0;
            if ((rc = om_rhs(m, &ps, U0, k1, NULL, NULL))) break;
            #pragma omp parallel for schedule(static)
            for (size_t i = 0; i < M; i++) U[i] = U0[i] + dt * k1[i];
        } else if (p->time_advance == 3103) { /* Kutta RK3 with the weights of Evolve.cpp:58-86 */
            ps.dsr_time = t0 + 0.0;
            if ((rc = om_rhs(m, &ps, U0, k1, NULL, NULL))) break;
            #pragma omp parallel for schedule(static)
            for (size_t i = 0; i < M; i++) Us[i] = U0[i] + 0.5 * dt * k1[i];
            ps.dsr_time = t0 + dt;
            if ((rc = om_rhs(m, &ps, Us, k2, NULL, NULL))) break;
            #pragma omp parallel for schedule(static)
            for (size_t i = 0; i < M; i++) Us[i] = U0[i] - dt * k1[i] + 2.0 * dt * k2[i];
            ps.dsr_time = t0 + 0.5 * dt;
            if ((rc = om_rhs(m, &ps, Us, k3, NULL, NULL))) break;
            const double dt_on_6 = dt / 6.0;
            #pragma omp parallel for schedule(static)
            for (size_t i = 0; i < M; i++) U[i] = U0[i] + dt_on_6 * (k1[i] + 4 * k2[i] + k3[i]);
        } else if (p->time_advance == 3104) { /* SSP-RK3 (Shu-Osher), new in this path */
            ps.dsr_time = t0 + 0.0;
            if ((rc = om_rhs(m, &ps, U0, k1, NULL, NULL))) break;
            #pragma omp parallel for schedule(static)
            for (size_t i = 0; i < M; i++) U1[i] = U0[i] + dt * k1[i];
            ps.dsr_time = t0 + dt;
            if ((rc = om_rhs(m, &ps, U1, k2, NULL, NULL))) break;
            #pragma omp parallel for schedule(static)
            for (size_t i = 0; i < M; i++) Us[i] = 0.75 * U0[i] + 0.25 * (U1[i] + dt * k2[i]);
            ps.dsr_time = t0 + 0.5 * dt;
            if ((rc = om_rhs(m, &ps, Us, k3, NULL, NULL))) break;
            #pragma omp parallel for schedule(static)
            for (size_t i = 0; i < M; i++) U[i] = (1.0 / 3.0) * U0[i] + (2.0 / 3.0) * (Us[i] + dt * k3[i]);
        } else {
            rc = -2;
            break;
        }
        int r = om_restrict(m, p, U); /* once per step, CIteration.cpp:79 */
        if (r < 0) { rc = r == -1 ? -9 : r; break; }
    }
    if (last_rhs && rc == 0) {
        const double* src = (p->time_advance == 3101) ? k1 : k3;
        memcpy(last_rhs, src, M * sizeof(double));
    }
    free(U0); free(k1); free(k2); free(k3); free(Us); free(U1);
    return rc;
}

/* host threads of the oracle's loops (n <= 0 leaves the count as it is); returns the count */
int om_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* get_residual_host, FVMR/src/output/residual/Residual.cpp:4-43 */
void om_residual(const om_mesh* m, const double* rhs, int norm, double* out) {
    const int N = m->N;
    for (int v = 0; v < 4; v++) {
        double s = 0;
        for (int i = 0; i < N; i++) {
            double f = m_abs(rhs[v * N + i]);
            if (norm == 1) s += f;
            else if (norm == 2) s += f * f;
            else s = m_max(s, f);
        }
        if (norm == 2) s = sqrt(s);
        out[v] = s;
    }
}

/* ---- field output ------------------------------------------------------- */

/* FieldWriter::update_nodeField_ruvp (FVMR/src/output/FieldWriter.cpp:370-402) over
 * CIteration::update_host_ruvp_Uold's U2ruvp (FVMR/src/time/CIteration.cpp:163-180),
 * then update_nodeField_other_variables (FieldWriter.cpp:404-430) and
 * ReferenceData::update_farfield (FieldWriter.cpp:540-549) for p_inf, pdyn_inf */
void om_node_field(int N, int V, const int* elem_nodes, const double* U, double gamma, double p_inf,
                   double pdyn_inf, double* out) {
    int* cnt = (int*)calloc((size_t)(V > 0 ? V : 1), sizeof(int));
    for (int k = 0; k < 4; k++) memset(out + (size_t)k * V, 0, sizeof(double) * (size_t)V);
    for (int e = 0; e < N; e++) {
        const double r = U[e], uu = U[(size_t)N + e] / U[e], vv = U[2 * (size_t)N + e] / U[e];
        const double pp = r * (gamma - 1) * (U[3 * (size_t)N + e] / U[e] - (uu * uu + vv * vv) * 0.5);
        const double ruvp[4] = {r, uu, vv, pp};
        for (int j = 0; j < 4; j++) {
            const int n = elem_nodes[(size_t)j * N + e];
            if (n < 0 || n >= V) continue;
            cnt[n]++;
            for (int k = 0; k < 4; k++) out[(size_t)k * V + n] += ruvp[k];
        }
    }
    for (int n = 0; n < V; n++) {
        if (cnt[n] != 0)
            for (int k = 0; k < 4; k++) out[(size_t)k * V + n] /= cnt[n];
        const double rho = out[n], u = out[(size_t)V + n], v = out[2 * (size_t)V + n], p = out[3 * (size_t)V + n];
        out[4 * (size_t)V + n] = (p - p_inf) / pdyn_inf;
        const double V2 = u * u + v * v;
        const double a2 = gamma * p / rho;
        out[5 * (size_t)V + n] = sqrt(V2 / a2);
    }
    free(cnt);
}

void om_boundary_forces(int NB, const int* set_off, const int* set_list, const int* bc_type, int E,
                        const int* edge_nodes, const double* edge_normal, const double* edge_len,
                        const double* Cp, double ref_area, double* cd, double* cl, double* cd_wall,
                        double* cl_wall) {
    const double one_on_Sref = 1 / ref_area;
    double dw = 0.0, lw = 0.0;
    for (int b = 0; b < NB; b++) {
        double CD = 0.0, CL = 0.0;
        for (int k = set_off[b]; k < set_off[b + 1]; k++) {
            const int e = set_list[k];
            const int n0 = edge_nodes[e], n1 = edge_nodes[(size_t)E + e];
            const double c = 0.5 * (Cp[n0] + Cp[n1]);
            const double dC = c * one_on_Sref * edge_len[e];
            CD += dC * edge_normal[e];
            CL += dC * edge_normal[(size_t)E + e];
        }
        cd[b] = CD;
        cl[b] = CL;
        /* _BC_wall_nonViscous, _BC_wall_adiabat, _BC_wall_isothermal (Constexpr.h:40-42) */
        if (bc_type[b] == 6001 || bc_type[b] == 6002 || bc_type[b] == 6003) {
            dw += CD;
            lw += CL;
        }
    }
    *cd_wall = dw;
    *cl_wall = lw;
}

/* getColor_device (CudaGrid_kernels.cu:24-66) with the map of CudaGrid.cpp:31-37 */
static void om_colour_of(float x, float* rgb) {
    static const float map[5][4] = {{1.0f, 0.0f, 0.0f, 0.00f}, {1.0f, 1.0f, 0.0f, 0.25f}, {0.0f, 1.0f, 0.0f, 0.50f},
                                    {0.0f, 0.0f, 1.0f, 0.75f}, {1.0f, 0.0f, 1.0f, 1.00f}};
    if (x < 0.0f) x = 0.0f;
    if (x > 1.0f) x = 1.0f;
    for (int i = 0; i < 4; i++) {
        if (x >= map[i][3] && x <= map[i + 1][3]) {
            const float t0 = map[i][3], t1 = map[i + 1][3];
            const float n = (x - t0) / (t1 - t0);
            const float omn = 1 - n;
            const float omn2 = omn * omn, omn3 = omn2 * omn;
            const float n2 = n * n, n3 = n2 * n;
            for (int k = 0; k < 3; k++) {
                const float c0 = map[i][k], c1 = map[i + 1][k];
                const float cm = 0.5f * (c0 + c1);
                rgb[k] = omn3 * c0 + 3 * omn2 * n * cm + 3 * omn * n2 * cm + n3 * c1;
            }
            return;
        }
    }
    rgb[0] = 252.0f / 255.0f;
    rgb[1] = 3.0f / 255.0f;
    rgb[2] = 253.0f / 255.0f;
}

/* accumulateElementDataToNodeData_k, divideNodeData_k, nodeDataToVertexColor_k
 * (CudaGrid_kernels.cu:79-130), run in cell order: the max it takes is the same in
 * any order except for NaN */
void om_colour_nodes(int N, int V, const int* elem_nodes, const double* U, float range_lo, float range_hi,
                     float* rgb, float* node_value) {
    int* cnt = (int*)calloc((size_t)(V > 0 ? V : 1), sizeof(int));
    for (int e = 0; e < N; e++)
        for (int j = 0; j < 3; j++) cnt[elem_nodes[(size_t)j * N + e]]++;
    for (int n = 0; n < V; n++) node_value[n] = 0.0f;
    for (int e = 0; e < N; e++)
        for (int j = 0; j < 3; j++) {
            const int n = elem_nodes[(size_t)j * N + e];
            float x = (float)U[e];
            x *= cnt[n];
            const float v = node_value[n];
            node_value[n] = (v > x) ? v : x;
        }
    for (int n = 0; n < V; n++) {
        float div = (float)(1.0 / cnt[n]);
        if (div > 1e5) div = 1.0f;
        node_value[n] *= div;
        const float len = fabsf(range_hi - range_lo);
        const float x = (len == 0) ? 0.0f : (node_value[n] - range_lo) / len;
        om_colour_of(x, rgb + 3 * (size_t)n);
    }
    free(cnt);
}
