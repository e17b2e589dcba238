/*
 * plk_oracle.c — CPU oracle for the LightningKokkos state-vector hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).  Each
 * routine restates one reference functor; the citation above it names the
 * file:line it follows (paths relative to the reference project root,
 * pennylane_lightning_kokkos/src/...).  The arithmetic keeps the functors'
 * operation order: Kokkos::complex products are (a.re*b.re - a.im*b.im,
 * a.re*b.im + a.im*b.re), scalar*complex scales both parts.  Build with
 * -ffp-contract=off so that x86 and Arm hosts give identical bits.
 */
#include "plk_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* complex helpers (Kokkos::complex semantics)                              */
/* ------------------------------------------------------------------------ */
static inline orc_cplx C(double re, double im) {
    orc_cplx z = {re, im};
    return z;
}
static inline orc_cplx cmul(orc_cplx a, orc_cplx b) {
    return C(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline orc_cplx cadd(orc_cplx a, orc_cplx b) {
    return C(a.re + b.re, a.im + b.im);
}
static inline orc_cplx csub(orc_cplx a, orc_cplx b) {
    return C(a.re - b.re, a.im - b.im);
}
static inline orc_cplx rmul(double s, orc_cplx a) { return C(s * a.re, s * a.im); }
static inline orc_cplx cconj(orc_cplx a) { return C(a.re, -a.im); }
/* Kokkos::exp(z) = exp(re) * (cos(im), sin(im)) */
static inline orc_cplx cexp_(orc_cplx z) {
    double e = exp(z.re);
    return C(e * cos(z.im), e * sin(z.im));
}
static inline void cswap(orc_cplx *a, orc_cplx *b) {
    orc_cplx t = *a;
    *a = *b;
    *b = t;
}

static int g_threads = 0;
void orc_set_num_threads(int n) { g_threads = n; }
int orc_get_num_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}
#define PAR_THRESHOLD (1ULL << 14)
#define OMP_FOR _Pragma("omp parallel for schedule(static) num_threads(orc_get_num_threads()) if (cnt >= PAR_THRESHOLD)")

/* ------------------------------------------------------------------------ */
/* index helpers (src/util/UtilKokkos.hpp:97-106)                           */
/* ------------------------------------------------------------------------ */
static inline uint64_t trailing_ones(int pos) {
    return (pos == 0) ? 0 : (~(uint64_t)0 >> (64 - pos));
}
static inline uint64_t leading_ones(int pos) {
    return (pos >= 64) ? 0 : (~(uint64_t)0 << pos);
}

/* Parity masks for m sorted bit positions, as the functors build them:
 * parity_low = fillTrailingOnes(p0), ..., middle masks
 * fillLeadingOnes(p_{j-1}+1) & fillTrailingOnes(p_j), parity_high =
 * fillLeadingOnes(p_{m-1}+1) (GateFunctors.hpp:96-101, :1380-1395,
 * :2020-2032).  The base index of group k is OR_j ((k << j) & mask_j). */
typedef struct {
    int m;
    uint64_t mask[5];
} orc_masks;

static void make_masks(const int *sorted, int m, orc_masks *out) {
    out->m = m;
    for (int j = 0; j <= m; j++) {
        uint64_t lo = (j == 0) ? ~(uint64_t)0 : leading_ones(sorted[j - 1] + 1);
        uint64_t hi = (j == m) ? ~(uint64_t)0 : trailing_ones(sorted[j]);
        out->mask[j] = lo & hi;
    }
}
static inline uint64_t base_index(uint64_t k, const orc_masks *mk) {
    uint64_t r = 0;
    for (int j = 0; j <= mk->m; j++) r |= (k << j) & mk->mask[j];
    return r;
}

static void sort_small(int *a, int m) {
    for (int i = 1; i < m; i++) {
        int v = a[i], j = i - 1;
        while (j >= 0 && a[j] > v) {
            a[j + 1] = a[j];
            j--;
        }
        a[j + 1] = v;
    }
}

/* wire lists hold at most ORC_MAX_QUBITS entries (every wire of the state) */
#define ORC_MAX_QUBITS 40

static int check_wires(int nq, const int64_t *wires, int nw) {
    if (nq < 1 || nq > ORC_MAX_QUBITS || nw < 1 || nw > nq) return ORC_BAD_ARGS;
    for (int i = 0; i < nw; i++) {
        if (wires[i] < 0 || wires[i] >= nq) return ORC_BAD_ARGS;
        for (int j = 0; j < i; j++)
            if (wires[i] == wires[j]) return ORC_BAD_ARGS;
    }
    return ORC_OK;
}

/* rev[j] = nq - wires[j] - 1 */
static void rev_wires(int nq, const int64_t *wires, int nw, int *rev) {
    for (int j = 0; j < nw; j++) rev[j] = nq - (int)wires[j] - 1;
}

/* ------------------------------------------------------------------------ */
/* gate kinds                                                               */
/* ------------------------------------------------------------------------ */
enum {
    G_X, G_Y, G_Z, G_H, G_S, G_T, G_PS, G_RX, G_RY, G_RZ, G_ROT,
    G_CNOT, G_CY, G_CZ, G_SWAP, G_CPS, G_CRX, G_CRY, G_CRZ, G_CROT,
    G_IXX, G_IXY, G_IYY, G_IZZ, G_SE, G_SEM, G_SEP,
    G_DE, G_DEM, G_DEP, G_CSWAP, G_TOF, G_MRZ, G_ID, G_UNKNOWN
};

static int gate_kind(const char *name) {
    static const struct {
        const char *n;
        int k;
    } tbl[] = {
        {"PauliX", G_X}, {"PauliY", G_Y}, {"PauliZ", G_Z}, {"Hadamard", G_H},
        {"S", G_S}, {"T", G_T}, {"PhaseShift", G_PS}, {"RX", G_RX},
        {"RY", G_RY}, {"RZ", G_RZ}, {"Rot", G_ROT}, {"CNOT", G_CNOT},
        {"CY", G_CY}, {"CZ", G_CZ}, {"SWAP", G_SWAP},
        {"ControlledPhaseShift", G_CPS}, {"CRX", G_CRX}, {"CRY", G_CRY},
        {"CRZ", G_CRZ}, {"CRot", G_CROT}, {"IsingXX", G_IXX},
        {"IsingXY", G_IXY}, {"IsingYY", G_IYY}, {"IsingZZ", G_IZZ},
        {"SingleExcitation", G_SE}, {"SingleExcitationMinus", G_SEM},
        {"SingleExcitationPlus", G_SEP}, {"DoubleExcitation", G_DE},
        {"DoubleExcitationMinus", G_DEM}, {"DoubleExcitationPlus", G_DEP},
        {"CSWAP", G_CSWAP}, {"Toffoli", G_TOF}, {"MultiRZ", G_MRZ},
        {"Identity", G_ID}};
    for (size_t i = 0; i < sizeof(tbl) / sizeof(tbl[0]); i++)
        if (strcmp(tbl[i].n, name) == 0) return tbl[i].k;
    return G_UNKNOWN;
}

static int gate_nwires(int kind) {
    switch (kind) {
    case G_X: case G_Y: case G_Z: case G_H: case G_S: case G_T: case G_PS:
    case G_RX: case G_RY: case G_RZ: case G_ROT:
        return 1;
    case G_CSWAP: case G_TOF:
        return 3;
    case G_DE: case G_DEM: case G_DEP:
        return 4;
    case G_MRZ: case G_ID:
        return -1; /* any */
    default:
        return 2;
    }
}

static int gate_nparams(int kind) {
    switch (kind) {
    case G_PS: case G_RX: case G_RY: case G_RZ: case G_CPS: case G_CRX:
    case G_CRY: case G_CRZ: case G_IXX: case G_IXY: case G_IYY: case G_IZZ:
    case G_SE: case G_SEM: case G_SEP: case G_DE: case G_DEM: case G_DEP:
    case G_MRZ:
        return 1;
    case G_ROT: case G_CROT:
        return 3;
    default:
        return 0;
    }
}

/* Rot / CRot matrix (GateFunctors.hpp:3134-3160 rotFunctor, :782-815
 * cRotFunctor): Rot = RZ(omega) RY(theta) RZ(phi); inverse negates and
 * reverses the angles. */
static void rot_matrix(const double *p, int inverse, orc_cplx m[4]) {
    const double phi = inverse ? -p[2] : p[0];
    const double theta = inverse ? -p[1] : p[1];
    const double omega = inverse ? -p[0] : p[2];
    const double c = cos(theta / 2), s = sin(theta / 2);
    const double pp = phi + omega, mm = phi - omega;
    const orc_cplx I = C(0.0, 1.0), mI = C(-0.0, -1.0);
    m[0] = rmul(c, cexp_(rmul(pp / 2, mI)));
    orc_cplx e01 = cexp_(rmul(mm / 2, I));
    m[1] = rmul(s, C(-e01.re, -e01.im));
    m[2] = rmul(s, cexp_(rmul(mm / 2, mI)));
    m[3] = rmul(c, cexp_(rmul(pp / 2, I)));
}

/* ------------------------------------------------------------------------ */
/* named gates                                                              */
/* ------------------------------------------------------------------------ */
int orc_apply(orc_cplx *a, int nq, const char *name, const int64_t *wires,
              int nw, int inverse, const double *params, int np) {
    const int kind = gate_kind(name);
    if (kind == G_UNKNOWN) return ORC_UNKNOWN_GATE;
    if (kind == G_ID) return ORC_OK; /* StateVectorKokkos.hpp:589-590 */
    const int need_w = gate_nwires(kind);
    if (need_w > 0 && nw != need_w) return ORC_BAD_ARGS;
    if (check_wires(nq, wires, nw) != ORC_OK) return ORC_BAD_ARGS;
    if (np < gate_nparams(kind)) return ORC_BAD_ARGS;
    const double th = (np > 0) ? params[0] : 0.0;
    int rev[ORC_MAX_QUBITS];
    rev_wires(nq, wires, nw, rev);

    if (kind == G_MRZ) {
        /* multiRZFunctor, GateFunctors.hpp:2132-2170 */
        const orc_cplx first = C(cos(th / 2), -sin(th / 2));
        const orc_cplx second = C(cos(th / 2), sin(th / 2));
        const orc_cplx s0 = inverse ? cconj(first) : first;
        const orc_cplx s1 = inverse ? cconj(second) : second;
        uint64_t par = 0;
        for (int j = 0; j < nw; j++) par |= (uint64_t)1 << rev[j];
        const uint64_t cnt = (uint64_t)1 << nq;
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++)
            a[k] = cmul(a[k], (__builtin_popcountll(k & par) % 2 == 0) ? s0 : s1);
        return ORC_OK;
    }

    if (nw == 1) {
        /* single-qubit functors, GateFunctors.hpp:302-647, 3134-3184 */
        const int r = rev[0];
        const uint64_t sh = (uint64_t)1 << r;
        const uint64_t par = trailing_ones(r), par_inv = leading_ones(r + 1);
        const uint64_t cnt = (uint64_t)1 << (nq - 1);
        orc_cplx c0 = C(0, 0), c1 = C(0, 0), m[4];
        double c = 0, s = 0;
        switch (kind) {
        case G_S: c0 = inverse ? C(-0.0, -1.0) : C(0.0, 1.0); break;
        case G_T: {
            orc_cplx e = cexp_(C(0, M_PI / 4));
            c0 = inverse ? cconj(e) : e;
            break;
        }
        case G_PS:
            c0 = inverse ? cexp_(C(-0.0, -th)) : cexp_(C(0.0, th));
            break;
        case G_RX:
            c = cos(th * 0.5);
            s = inverse ? sin(th * 0.5) : sin(-th * 0.5);
            break;
        case G_RY:
            c = cos(th * 0.5);
            s = inverse ? -sin(th * 0.5) : sin(th * 0.5);
            break;
        case G_RZ: {
            const double ca = cos(th * 0.5), sa = sin(th * 0.5);
            const orc_cplx f = C(ca, -sa), g = C(ca, sa);
            c0 = inverse ? cconj(f) : f;
            c1 = inverse ? cconj(g) : g;
            break;
        }
        case G_ROT: rot_matrix(params, inverse, m); break;
        default: break;
        }
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i0 = ((k << 1) & par_inv) | (par & k);
            const uint64_t i1 = i0 | sh;
            const orc_cplx v0 = a[i0], v1 = a[i1];
            switch (kind) {
            case G_X: a[i0] = v1; a[i1] = v0; break;
            case G_Y:
                a[i0] = C(v1.im, -v1.re);
                a[i1] = C(-v0.im, v0.re);
                break;
            case G_Z: a[i1] = rmul(-1.0, v1); break;
            case G_H:
                a[i0] = cadd(rmul(M_SQRT1_2, v0), rmul(M_SQRT1_2, v1));
                a[i1] = cadd(rmul(M_SQRT1_2, v0), rmul(-M_SQRT1_2, v1));
                break;
            case G_S: case G_T: case G_PS: a[i1] = cmul(v1, c0); break;
            case G_RX:
                a[i0] = cadd(rmul(c, v0), C(-v1.im * s, v1.re * s));
                a[i1] = cadd(C(-v0.im * s, v0.re * s), rmul(c, v1));
                break;
            case G_RY:
                a[i0] = C(c * v0.re - s * v1.re, c * v0.im - s * v1.im);
                a[i1] = C(s * v0.re + c * v1.re, s * v0.im + c * v1.im);
                break;
            case G_RZ:
                a[i0] = cmul(v0, c0);
                a[i1] = cmul(v1, c1);
                break;
            case G_ROT:
                a[i0] = cadd(cmul(m[0], v0), cmul(m[1], v1));
                a[i1] = cadd(cmul(m[2], v0), cmul(m[3], v1));
                break;
            default: break;
            }
        }
        return ORC_OK;
    }

    if (nw == 2) {
        /* two-qubit functors, GateFunctors.hpp:649-1340, 1769-1993;
         * rev_wire0 = target (wires[1]), rev_wire1 = control (wires[0]) */
        const int r0 = rev[1], r1 = rev[0];
        const uint64_t s0 = (uint64_t)1 << r0, s1 = (uint64_t)1 << r1;
        int srt[2] = {r0 < r1 ? r0 : r1, r0 < r1 ? r1 : r0};
        orc_masks mk;
        make_masks(srt, 2, &mk);
        const uint64_t cnt = (uint64_t)1 << (nq - 2);
        double c = cos(th / 2), s = inverse ? -sin(th / 2) : sin(th / 2);
        orc_cplx e0 = C(0, 0), e1 = C(0, 0), m[4];
        switch (kind) {
        case G_CPS:
            e0 = inverse ? cexp_(C(-0.0, -th)) : cexp_(C(0.0, th));
            break;
        case G_CRZ: case G_IZZ: {
            const orc_cplx f = C(cos(th / 2), -sin(th / 2));
            const orc_cplx g = C(cos(th / 2), sin(th / 2));
            e0 = inverse ? cconj(f) : f;
            e1 = inverse ? cconj(g) : g;
            break;
        }
        case G_SEM:
            e0 = inverse ? cexp_(C(0.0, th / 2)) : cexp_(C(0.0, -th / 2));
            break;
        case G_SEP:
            e0 = inverse ? cexp_(C(0.0, -th / 2)) : cexp_(C(0.0, th / 2));
            break;
        case G_CROT: rot_matrix(params, inverse, m); break;
        default: break;
        }
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i00 = base_index(k, &mk);
            const uint64_t i10 = i00 | s1, i01 = i00 | s0, i11 = i00 | s0 | s1;
            const orc_cplx v00 = a[i00], v01 = a[i01], v10 = a[i10], v11 = a[i11];
            switch (kind) {
            case G_CNOT: a[i10] = v11; a[i11] = v10; break;
            case G_CY:
                a[i10] = C(v11.im, -v11.re);
                a[i11] = C(-v10.im, v10.re);
                break;
            case G_CZ: a[i11] = rmul(-1.0, v11); break;
            case G_SWAP: a[i10] = v01; a[i01] = v10; break;
            case G_CPS: a[i11] = cmul(v11, e0); break;
            case G_CRX:
                a[i10] = C(c * v10.re + s * v11.im, c * v10.im - s * v11.re);
                a[i11] = C(c * v11.re + s * v10.im, c * v11.im - s * v10.re);
                break;
            case G_CRY:
                a[i10] = csub(rmul(c, v10), rmul(s, v11));
                a[i11] = cadd(rmul(s, v10), rmul(c, v11));
                break;
            case G_CRZ:
                a[i10] = cmul(v10, e0);
                a[i11] = cmul(v11, e1);
                break;
            case G_CROT:
                a[i10] = cadd(cmul(m[0], v10), cmul(m[1], v11));
                a[i11] = cadd(cmul(m[2], v10), cmul(m[3], v11));
                break;
            case G_IXX:
                a[i00] = C(c * v00.re + s * v11.im, c * v00.im - s * v11.re);
                a[i01] = C(c * v01.re + s * v10.im, c * v01.im - s * v10.re);
                a[i10] = C(c * v10.re + s * v01.im, c * v10.im - s * v01.re);
                a[i11] = C(c * v11.re + s * v00.im, c * v11.im - s * v00.re);
                break;
            case G_IXY:
                a[i01] = C(c * v01.re - s * v10.im, c * v01.im + s * v10.re);
                a[i10] = C(c * v10.re - s * v01.im, c * v10.im + s * v01.re);
                break;
            case G_IYY:
                a[i00] = C(c * v00.re - s * v11.im, c * v00.im + s * v11.re);
                a[i01] = C(c * v01.re + s * v10.im, c * v01.im - s * v10.re);
                a[i10] = C(c * v10.re + s * v01.im, c * v10.im - s * v01.re);
                a[i11] = C(c * v11.re - s * v00.im, c * v11.im + s * v00.re);
                break;
            case G_IZZ:
                a[i00] = cmul(v00, e0);
                a[i01] = cmul(v01, e1);
                a[i10] = cmul(v10, e1);
                a[i11] = cmul(v11, e0);
                break;
            case G_SE: case G_SEM: case G_SEP:
                if (kind != G_SE) {
                    a[i00] = cmul(v00, e0);
                    a[i11] = cmul(v11, e0);
                }
                a[i01] = csub(rmul(c, v01), rmul(s, v10));
                a[i10] = cadd(rmul(s, v01), rmul(c, v10));
                break;
            default: break;
            }
        }
        return ORC_OK;
    }

    if (nw == 3) {
        /* cSWAPFunctor :1995-2061, toffoliFunctor :2063-2130;
         * rev_wire2 = control wires[0], rev_wire1 = wires[1],
         * rev_wire0 = wires[2] */
        const uint64_t s0 = (uint64_t)1 << rev[2], s1 = (uint64_t)1 << rev[1],
                       s2 = (uint64_t)1 << rev[0];
        int srt[3] = {rev[0], rev[1], rev[2]};
        sort_small(srt, 3);
        orc_masks mk;
        make_masks(srt, 3, &mk);
        const uint64_t cnt = (uint64_t)1 << (nq - 3);
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i000 = base_index(k, &mk);
            if (kind == G_CSWAP) {
                cswap(&a[i000 | s2 | s0], &a[i000 | s2 | s1]);
            } else {
                cswap(&a[i000 | s2 | s1 | s0], &a[i000 | s2 | s1]);
            }
        }
        return ORC_OK;
    }

    if (nw == 4) {
        /* doubleExcitation(Minus|Plus)Functor :1343-1767;
         * rev_wire3 = wires[0], rev_wire2 = wires[1], rev_wire1 = wires[2],
         * rev_wire0 = wires[3].  The functors sort the four bit positions
         * with an explicit case analysis; the result is the sorted order. */
        const uint64_t s0 = (uint64_t)1 << rev[3], s1 = (uint64_t)1 << rev[2],
                       s2 = (uint64_t)1 << rev[1], s3 = (uint64_t)1 << rev[0];
        int srt[4] = {rev[0], rev[1], rev[2], rev[3]};
        sort_small(srt, 4);
        orc_masks mk;
        make_masks(srt, 4, &mk);
        const double cr = cos(th / 2), sj = inverse ? -sin(th / 2) : sin(th / 2);
        orc_cplx e = C(1, 0);
        if (kind == G_DEM) e = inverse ? cexp_(C(0.0, th / 2)) : cexp_(C(0.0, -th / 2));
        if (kind == G_DEP) e = inverse ? cexp_(C(0.0, -th / 2)) : cexp_(C(0.0, th / 2));
        const uint64_t cnt = (uint64_t)1 << (nq - 4);
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i0000 = base_index(k, &mk);
            const uint64_t i0011 = i0000 | s1 | s0, i1100 = i0000 | s3 | s2;
            const orc_cplx v3 = a[i0011], v12 = a[i1100];
            if (kind != G_DE) {
                for (int b = 0; b < 16; b++) {
                    if (b == 3 || b == 12) continue;
                    uint64_t idx = i0000 | ((b & 1) ? s0 : 0) | ((b & 2) ? s1 : 0) |
                                   ((b & 4) ? s2 : 0) | ((b & 8) ? s3 : 0);
                    a[idx] = cmul(a[idx], e);
                }
            }
            a[i0011] = csub(rmul(cr, v3), rmul(sj, v12));
            a[i1100] = cadd(rmul(sj, v3), rmul(cr, v12));
        }
        return ORC_OK;
    }
    return ORC_BAD_ARGS;
}

/* ------------------------------------------------------------------------ */
/* dense matrices                                                           */
/* ------------------------------------------------------------------------ */
/* singleQubitOpFunctor GateFunctors.hpp:15-66, twoQubitOpFunctor :77-193;
 * k >= 3: U applied on the requested wires, wires[0] the most significant
 * bit of the matrix row/column index. */
int orc_apply_matrix(orc_cplx *a, int nq, const orc_cplx *mat,
                     const int64_t *wires, int nw, int inverse) {
    if (check_wires(nq, wires, nw) != ORC_OK || nw > 12) return ORC_BAD_ARGS;
    int rev[ORC_MAX_QUBITS];
    rev_wires(nq, wires, nw, rev);
    const uint64_t dim = (uint64_t)1 << nw;
    if (nw == 1) {
        const int r = rev[0];
        const uint64_t sh = (uint64_t)1 << r, par = trailing_ones(r),
                       par_inv = leading_ones(r + 1), cnt = (uint64_t)1 << (nq - 1);
        orc_cplx m[4];
        for (int i = 0; i < 4; i++) m[i] = mat[i];
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i0 = ((k << 1) & par_inv) | (par & k), i1 = i0 | sh;
            const orc_cplx v0 = a[i0], v1 = a[i1];
            if (inverse) {
                a[i0] = cadd(cmul(cconj(m[0]), v0), cmul(cconj(m[2]), v1));
                a[i1] = cadd(cmul(cconj(m[1]), v0), cmul(cconj(m[3]), v1));
            } else {
                a[i0] = cadd(cmul(m[0], v0), cmul(m[1], v1));
                a[i1] = cadd(cmul(m[2], v0), cmul(m[3], v1));
            }
        }
        return ORC_OK;
    }
    if (nw == 2) {
        const int r0 = rev[1], r1 = rev[0];
        const uint64_t s0 = (uint64_t)1 << r0, s1 = (uint64_t)1 << r1;
        int srt[2] = {r0 < r1 ? r0 : r1, r0 < r1 ? r1 : r0};
        orc_masks mk;
        make_masks(srt, 2, &mk);
        const uint64_t cnt = (uint64_t)1 << (nq - 2);
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i00 = base_index(k, &mk);
            const uint64_t idx[4] = {i00, i00 | s0, i00 | s1, i00 | s0 | s1};
            orc_cplx v[4], o[4];
            for (int j = 0; j < 4; j++) v[j] = a[idx[j]];
            for (int row = 0; row < 4; row++) {
                /* sum in column order, as the functor's expression does */
                orc_cplx acc;
                if (inverse) {
                    acc = cmul(cconj(mat[0 * 4 + row]), v[0]);
                    for (int col = 1; col < 4; col++)
                        acc = cadd(acc, cmul(cconj(mat[col * 4 + row]), v[col]));
                } else {
                    acc = cmul(mat[row * 4 + 0], v[0]);
                    for (int col = 1; col < 4; col++)
                        acc = cadd(acc, cmul(mat[row * 4 + col], v[col]));
                }
                o[row] = acc;
            }
            for (int j = 0; j < 4; j++) a[idx[j]] = o[j];
        }
        return ORC_OK;
    }
    /* k >= 3 */
    int srt[16];
    for (int j = 0; j < nw; j++) srt[j] = rev[j];
    sort_small(srt, nw);
    uint64_t offs[4096];
    for (uint64_t i = 0; i < dim; i++) {
        uint64_t o = 0;
        for (int j = 0; j < nw; j++)
            if ((i >> (nw - 1 - j)) & 1) o |= (uint64_t)1 << rev[j];
        offs[i] = o;
    }
    const uint64_t cnt = (uint64_t)1 << (nq - nw);
    int ok = ORC_OK;
#pragma omp parallel num_threads(orc_get_num_threads()) if (cnt >= 1024)
    {
        orc_cplx *v = (orc_cplx *)malloc(sizeof(orc_cplx) * dim);
        if (!v) ok = ORC_BAD_ARGS;
#pragma omp for schedule(static)
        for (uint64_t k = 0; k < cnt; k++) {
            if (!v) continue;
            uint64_t base = 0, rem = k;
            /* insert zero bits at the sorted target positions */
            {
                uint64_t r = rem;
                for (int j = 0; j < nw; j++) {
                    const uint64_t lowmask = ((uint64_t)1 << srt[j]) - 1;
                    r = ((r & ~lowmask) << 1) | (r & lowmask);
                }
                base = r;
            }
            for (uint64_t i = 0; i < dim; i++) v[i] = a[base | offs[i]];
            for (uint64_t i = 0; i < dim; i++) {
                orc_cplx acc = C(0, 0);
                for (uint64_t j = 0; j < dim; j++) {
                    const orc_cplx mij = inverse ? cconj(mat[j * dim + i]) : mat[i * dim + j];
                    acc = cadd(acc, cmul(mij, v[j]));
                }
                a[base | offs[i]] = acc;
            }
        }
        free(v);
    }
    return ok;
}

/* multiQubitOpFunctor's own index map, GateFunctors.hpp:195-300: the
 * amplitude index of row `inner` of team `t` is (t*dim | inner) with, for
 * pos = 0..k-1 in order, bit (k-1-pos) swapped with bit rev_wire(pos). */
int orc_apply_matrix_refmap(orc_cplx *a, int nq, const orc_cplx *mat,
                            const int64_t *wires, int nw, int inverse) {
    if (check_wires(nq, wires, nw) != ORC_OK || nw > 12) return ORC_BAD_ARGS;
    const uint64_t dim = (uint64_t)1 << nw, cnt = (uint64_t)1 << (nq - nw);
    orc_cplx *v = (orc_cplx *)malloc(sizeof(orc_cplx) * dim);
    uint64_t *ind = (uint64_t *)malloc(sizeof(uint64_t) * dim);
    if (!v || !ind) {
        free(v);
        free(ind);
        return ORC_BAD_ARGS;
    }
    for (uint64_t t = 0; t < cnt; t++) {
        const uint64_t kk = t * dim;
        for (uint64_t inner = 0; inner < dim; inner++) {
            uint64_t idx = kk | inner;
            for (int pos = 0; pos < nw; pos++) {
                const int b1 = nw - pos - 1, b2 = nq - (int)wires[pos] - 1;
                const uint64_t x = ((idx >> b1) ^ (idx >> b2)) & 1;
                idx = idx ^ ((x << b1) | (x << b2));
            }
            ind[inner] = idx;
            v[inner] = a[idx];
        }
        for (uint64_t i = 0; i < dim; i++) {
            orc_cplx acc = C(0, 0);
            for (uint64_t j = 0; j < dim; j++) {
                const orc_cplx mij = inverse ? cconj(mat[j * dim + i]) : mat[i * dim + j];
                acc = cadd(acc, cmul(mij, v[j]));
            }
            a[ind[i]] = acc;
        }
    }
    free(v);
    free(ind);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* generators (StateVectorKokkos.hpp:1275-1580, GateFunctors.hpp:2172-3132) */
/* ------------------------------------------------------------------------ */
static double gen_scale(int kind) {
    switch (kind) {
    case G_PS: case G_CPS: return 1.0;
    case G_IXY: case G_DEP: return 0.5;
    default: return -0.5;
    }
}

double orc_apply_generator(orc_cplx *a, int nq, const char *name,
                           const int64_t *wires, int nw, int adj, int *status) {
    (void)adj; /* the generator functors ignore their adj flag */
    int kind = gate_kind(name);
    *status = ORC_OK;
    switch (kind) {
    case G_RX: case G_RY: case G_RZ: {
        /* applyGeneratorRX/RY/RZ apply PauliX/Y/Z, :1452-1488 */
        const char *pn = kind == G_RX ? "PauliX" : (kind == G_RY ? "PauliY" : "PauliZ");
        *status = orc_apply(a, nq, pn, wires, nw, 0, NULL, 0);
        return -0.5;
    }
    case G_PS: case G_IXX: case G_IXY: case G_IYY: case G_IZZ: case G_SE:
    case G_SEM: case G_SEP: case G_DE: case G_DEM: case G_DEP: case G_CPS:
    case G_CRX: case G_CRY: case G_CRZ: case G_MRZ:
        break;
    default:
        *status = ORC_UNKNOWN_GATE;
        return 0.0;
    }
    if (check_wires(nq, wires, nw) != ORC_OK ||
        (kind != G_MRZ && gate_nwires(kind) != nw)) {
        *status = ORC_BAD_ARGS;
        return 0.0;
    }
    int rev[ORC_MAX_QUBITS];
    rev_wires(nq, wires, nw, rev);
    const orc_cplx Z0 = C(0.0, 0.0), PI_ = C(0.0, 1.0), MI_ = C(0.0, -1.0);
    if (kind == G_MRZ) {
        /* generatorMultiRZFunctor :3110-3132 */
        uint64_t par = 0;
        for (int j = 0; j < nw; j++) par |= (uint64_t)1 << rev[j];
        const uint64_t cnt = (uint64_t)1 << nq;
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++)
            a[k] = rmul((double)(1 - 2 * (int)(__builtin_popcountll(k & par) % 2)), a[k]);
        return -0.5;
    }
    if (kind == G_PS) {
        /* generatorPhaseShiftFunctor :2172-2198 */
        const int r = rev[0];
        const uint64_t par = trailing_ones(r), par_inv = leading_ones(r + 1),
                       cnt = (uint64_t)1 << (nq - 1);
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++) a[((k << 1) & par_inv) | (par & k)] = Z0;
        return 1.0;
    }
    if (nw == 2) {
        const int r0 = rev[1], r1 = rev[0];
        const uint64_t s0 = (uint64_t)1 << r0, s1 = (uint64_t)1 << r1;
        int srt[2] = {r0 < r1 ? r0 : r1, r0 < r1 ? r1 : r0};
        orc_masks mk;
        make_masks(srt, 2, &mk);
        const uint64_t cnt = (uint64_t)1 << (nq - 2);
        OMP_FOR
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i00 = base_index(k, &mk);
            const uint64_t i01 = i00 | s0, i10 = i00 | s1, i11 = i00 | s0 | s1;
            switch (kind) {
            case G_IXX: /* :2200-2246 */
                cswap(&a[i00], &a[i11]);
                cswap(&a[i10], &a[i01]);
                break;
            case G_IXY: /* :2248-2295 */
                cswap(&a[i10], &a[i01]);
                a[i00] = Z0;
                a[i11] = Z0;
                break;
            case G_IYY: { /* :2297-2345 */
                const orc_cplx v00 = a[i00];
                a[i00] = rmul(-1.0, a[i11]);
                a[i11] = rmul(-1.0, v00);
                cswap(&a[i10], &a[i01]);
                break;
            }
            case G_IZZ: /* :2347-2392 */
                a[i10] = rmul(-1.0, a[i10]);
                a[i01] = rmul(-1.0, a[i01]);
                break;
            case G_SE: /* :2394-2445 */
                a[i00] = Z0;
                a[i01] = cmul(a[i01], PI_);
                a[i10] = cmul(a[i10], MI_);
                a[i11] = Z0;
                cswap(&a[i10], &a[i01]);
                break;
            case G_SEM: /* :2447-2495 */
                a[i01] = cmul(a[i01], PI_);
                a[i10] = cmul(a[i10], MI_);
                cswap(&a[i10], &a[i01]);
                break;
            case G_SEP: /* :2497-2549 */
                a[i00] = rmul(-1.0, a[i00]);
                a[i01] = cmul(a[i01], PI_);
                a[i10] = cmul(a[i10], MI_);
                a[i11] = rmul(-1.0, a[i11]);
                cswap(&a[i10], &a[i01]);
                break;
            case G_CPS: /* :2914-2959 */
                a[i00] = Z0;
                a[i01] = Z0;
                a[i10] = Z0;
                break;
            case G_CRX: /* :2961-3007 */
                a[i00] = Z0;
                a[i01] = Z0;
                cswap(&a[i10], &a[i11]);
                break;
            case G_CRY: { /* :3009-3060 */
                a[i00] = Z0;
                a[i01] = Z0;
                const orc_cplx v0 = a[i10];
                a[i10] = C(a[i11].im, -a[i11].re);
                a[i11] = C(-v0.im, v0.re);
                break;
            }
            case G_CRZ: /* :3062-3108 */
                a[i00] = Z0;
                a[i01] = Z0;
                a[i11] = rmul(-1.0, a[i11]);
                break;
            default: break;
            }
        }
        return gen_scale(kind);
    }
    /* 4-qubit: generatorDoubleExcitation(Minus|Plus)Functor :2551-2912 */
    const uint64_t s0 = (uint64_t)1 << rev[3], s1 = (uint64_t)1 << rev[2],
                   s2 = (uint64_t)1 << rev[1], s3 = (uint64_t)1 << rev[0];
    int srt[4] = {rev[0], rev[1], rev[2], rev[3]};
    sort_small(srt, 4);
    orc_masks mk;
    make_masks(srt, 4, &mk);
    const uint64_t cnt = (uint64_t)1 << (nq - 4);
    OMP_FOR
    for (uint64_t k = 0; k < cnt; k++) {
        const uint64_t i0000 = base_index(k, &mk);
        const uint64_t i0011 = i0000 | s1 | s0, i1100 = i0000 | s3 | s2;
        if (kind == G_DE) {
            const orc_cplx v3 = a[i0011], v12 = a[i1100];
            for (int b = 0; b < 16; b++) {
                uint64_t idx = i0000 | ((b & 1) ? s0 : 0) | ((b & 2) ? s1 : 0) |
                               ((b & 4) ? s2 : 0) | ((b & 8) ? s3 : 0);
                a[idx] = Z0;
            }
            a[i0011] = cmul(v12, MI_);
            a[i1100] = cmul(v3, PI_);
        } else if (kind == G_DEM) {
            a[i0011] = cmul(a[i0011], PI_);
            a[i1100] = cmul(a[i1100], MI_);
            cswap(&a[i1100], &a[i0011]);
        } else {
            a[i0011] = cmul(a[i0011], MI_);
            a[i1100] = cmul(a[i1100], PI_);
            cswap(&a[i1100], &a[i0011]);
        }
    }
    return gen_scale(kind);
}

/* ------------------------------------------------------------------------ */
/* expectation values (ExpValFunctors.hpp, MeasuresKokkos.hpp:80-346)       */
/* ------------------------------------------------------------------------ */
#define OMP_RED _Pragma("omp parallel for schedule(static) reduction(+ : acc) num_threads(orc_get_num_threads()) if (cnt >= PAR_THRESHOLD)")

double orc_expval_named(const orc_cplx *a, int nq, const char *name,
                        const int64_t *wires, int nw, int *status) {
    *status = ORC_OK;
    double acc = 0.0;
    if (strcmp(name, "Identity") == 0) {
        /* getExpectationValueIdentityFunctor :13-28 */
        const uint64_t cnt = (uint64_t)1 << nq;
        OMP_RED
        for (uint64_t k = 0; k < cnt; k++) acc += a[k].re * a[k].re + a[k].im * a[k].im;
        return acc;
    }
    if (nw != 1 || check_wires(nq, wires, nw) != ORC_OK) {
        *status = ORC_BAD_ARGS;
        return 0.0;
    }
    const int r = nq - (int)wires[0] - 1;
    const uint64_t sh = (uint64_t)1 << r, par = trailing_ones(r),
                   par_inv = leading_ones(r + 1), cnt = (uint64_t)1 << (nq - 1);
    int which = -1;
    if (strcmp(name, "PauliX") == 0) which = 0;
    else if (strcmp(name, "PauliY") == 0) which = 1;
    else if (strcmp(name, "PauliZ") == 0) which = 2;
    else if (strcmp(name, "Hadamard") == 0) which = 3;
    if (which < 0) {
        *status = ORC_UNKNOWN_GATE;
        return 0.0;
    }
    OMP_RED
    for (uint64_t k = 0; k < cnt; k++) {
        const uint64_t i0 = ((k << 1) & par_inv) | (par & k), i1 = i0 | sh;
        const orc_cplx v0 = a[i0], v1 = a[i1];
        switch (which) {
        case 0: /* :30-58: Re(conj(v0) v1) + Re(conj(v1) v0) */
            acc += cmul(cconj(v0), v1).re;
            acc += cmul(cconj(v1), v0).re;
            break;
        case 1: /* :60-92 */
            acc += cmul(cconj(v0), C(v1.im, -v1.re)).re;
            acc += cmul(cconj(v1), C(-v0.im, v0.re)).re;
            break;
        case 2: /* :94-121 */
            acc += cmul(cconj(v1), rmul(-1.0, v1)).re;
            acc += cmul(cconj(v0), v0).re;
            break;
        default: { /* :123-153 */
            orc_cplx t = cadd(cmul(cconj(v0), cadd(v0, v1)), cmul(cconj(v1), csub(v0, v1)));
            acc += rmul(M_SQRT1_2, t).re;
        }
        }
    }
    return acc;
}

double orc_inner_re(const orc_cplx *x, const orc_cplx *y, size_t n) {
    /* getRealOfComplexInnerProductFunctor LinearAlgebraKokkos.hpp:155-192 */
    double acc = 0.0;
    const uint64_t cnt = n;
    OMP_RED
    for (uint64_t k = 0; k < cnt; k++) acc += x[k].re * y[k].re + x[k].im * y[k].im;
    return acc;
}

double orc_inner_im(const orc_cplx *x, const orc_cplx *y, size_t n) {
    /* getImagOfComplexInnerProductFunctor LinearAlgebraKokkos.hpp:199-236 */
    double acc = 0.0;
    const uint64_t cnt = n;
    OMP_RED
    for (uint64_t k = 0; k < cnt; k++) acc += x[k].re * y[k].im - x[k].im * y[k].re;
    return acc;
}

double orc_expval_matrix(const orc_cplx *a, int nq, const orc_cplx *mat,
                         const int64_t *wires, int nw, int *status) {
    *status = ORC_OK;
    if (check_wires(nq, wires, nw) != ORC_OK) {
        *status = ORC_BAD_ARGS;
        return 0.0;
    }
    double acc = 0.0;
    if (nw == 1) {
        /* getExpectationValueSingleQubitOpFunctor :155-188 */
        const int r = nq - (int)wires[0] - 1;
        const uint64_t sh = (uint64_t)1 << r, par = trailing_ones(r),
                       par_inv = leading_ones(r + 1), cnt = (uint64_t)1 << (nq - 1);
        OMP_RED
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i0 = ((k << 1) & par_inv) | (par & k), i1 = i0 | sh;
            const orc_cplx v0 = a[i0], v1 = a[i1];
            orc_cplx t = cadd(cmul(cconj(v0), cadd(cmul(mat[0], v0), cmul(mat[1], v1))),
                              cmul(cconj(v1), cadd(cmul(mat[2], v0), cmul(mat[3], v1))));
            acc += t.re;
        }
        return acc;
    }
    if (nw == 2) {
        /* getExpectationValueTwoQubitOpFunctor :190-250 */
        const int r0 = nq - (int)wires[1] - 1, r1 = nq - (int)wires[0] - 1;
        const uint64_t s0 = (uint64_t)1 << r0, s1 = (uint64_t)1 << r1;
        int srt[2] = {r0 < r1 ? r0 : r1, r0 < r1 ? r1 : r0};
        orc_masks mk;
        make_masks(srt, 2, &mk);
        const uint64_t cnt = (uint64_t)1 << (nq - 2);
        OMP_RED
        for (uint64_t k = 0; k < cnt; k++) {
            const uint64_t i00 = base_index(k, &mk);
            const uint64_t idx[4] = {i00, i00 | s0, i00 | s1, i00 | s0 | s1};
            orc_cplx v[4], t = C(0, 0);
            for (int j = 0; j < 4; j++) v[j] = a[idx[j]];
            for (int row = 0; row < 4; row++) {
                orc_cplx mv = cmul(mat[row * 4], v[0]);
                for (int col = 1; col < 4; col++) mv = cadd(mv, cmul(mat[row * 4 + col], v[col]));
                t = row == 0 ? cmul(cconj(v[0]), mv) : cadd(t, cmul(cconj(v[row]), mv));
            }
            acc += t.re;
        }
        return acc;
    }
    /* k >= 3: copy, apply the matrix, Re<psi|M psi> (MeasuresKokkos.hpp:339-345) */
    const size_t n = (size_t)1 << nq;
    orc_cplx *tmp = (orc_cplx *)malloc(sizeof(orc_cplx) * n);
    if (!tmp) {
        *status = ORC_BAD_ARGS;
        return 0.0;
    }
    memcpy(tmp, a, sizeof(orc_cplx) * n);
    *status = orc_apply_matrix(tmp, nq, mat, wires, nw, 0);
    double r = orc_inner_re(a, tmp, n);
    free(tmp);
    return r;
}

double orc_expval_sparse(const orc_cplx *a, int64_t nrows, const orc_cplx *data,
                         const int64_t *indices, const int64_t *indptr) {
    /* getExpectationValueSparseFunctor ExpValFunctors.hpp:252-280 */
    double acc = 0.0;
    const uint64_t cnt = (uint64_t)nrows;
    OMP_RED
    for (uint64_t row = 0; row < cnt; row++) {
        for (int64_t j = indptr[row]; j < indptr[row + 1]; j++)
            acc += cmul(cmul(cconj(a[row]), data[j]), a[indices[j]]).re;
    }
    return acc;
}

void orc_axpy(orc_cplx alpha, const orc_cplx *x, orc_cplx *y, size_t n) {
    /* axpy_KokkosFunctor LinearAlgebraKokkos.hpp:30-47 */
    const uint64_t cnt = n;
    OMP_FOR
    for (uint64_t k = 0; k < cnt; k++) y[k] = cadd(y[k], cmul(alpha, x[k]));
}

void orc_spmv(const orc_cplx *x, orc_cplx *y, int64_t nrows, const orc_cplx *data,
              const int64_t *indices, const int64_t *indptr) {
    /* SparseMV_KokkosFunctor LinearAlgebraKokkos.hpp:68-104 */
    const uint64_t cnt = (uint64_t)nrows;
    OMP_FOR
    for (uint64_t row = 0; row < cnt; row++) {
        orc_cplx t = C(0.0, 0.0);
        for (int64_t j = indptr[row]; j < indptr[row + 1]; j++)
            t = cadd(t, cmul(data[j], x[indices[j]]));
        y[row] = t;
    }
}

/* ------------------------------------------------------------------------ */
/* probabilities and sampling                                               */
/* ------------------------------------------------------------------------ */
void orc_probs(const orc_cplx *a, int nq, double *out) {
    /* getProbFunctor MeasuresFunctors.hpp:15-30 */
    const uint64_t cnt = (uint64_t)1 << nq;
    OMP_FOR
    for (uint64_t k = 0; k < cnt; k++) out[k] = a[k].re * a[k].re + a[k].im * a[k].im;
}

int orc_probs_wires(const orc_cplx *a, int nq, const int64_t *wires, int nw,
                    double *out) {
    /* MeasuresKokkos::probs(wires) :418-517: marginal over the sorted wires
     * (getSubProbFunctor, generateBitsPatterns), then transposed to the
     * requested order (getTransposedIndexFunctor / getTransposedFunctor). */
    if (check_wires(nq, wires, nw) != ORC_OK) return ORC_BAD_ARGS;
    int64_t sorted_w[64];
    int order[64];
    for (int i = 0; i < nw; i++) order[i] = i;
    for (int i = 1; i < nw; i++) { /* stable argsort */
        int v = order[i], j = i - 1;
        while (j >= 0 && wires[order[j]] > wires[v]) {
            order[j + 1] = order[j];
            j--;
        }
        order[j + 1] = v;
    }
    for (int i = 0; i < nw; i++) sorted_w[i] = wires[order[i]];
    const uint64_t nout = (uint64_t)1 << nw;
    double *sub = (double *)calloc(nout, sizeof(double));
    if (!sub) return ORC_BAD_ARGS;
    /* index = pattern(sorted wires) + pattern(other wires); sorted wire j
     * (j = 0 most significant) is bit (nw-1-j) of the output index. */
    for (uint64_t idx = 0; idx < ((uint64_t)1 << nq); idx++) {
        uint64_t o = 0;
        for (int j = 0; j < nw; j++)
            o |= ((idx >> (nq - 1 - sorted_w[j])) & 1) << (nw - 1 - j);
        sub[o] += a[idx].re * a[idx].re + a[idx].im * a[idx].im;
    }
    /* trans_index[i] = sum_j ((i >> (nw-1-j)) & 1) << (nw-1-order[j]) */
    for (uint64_t i = 0; i < nout; i++) {
        uint64_t t = 0;
        for (int j = 0; j < nw; j++) {
            const uint64_t bit = (i >> (nw - 1 - j)) & 1;
            t += bit << (nw - 1 - order[j]);
        }
        out[i] = sub[t];
    }
    free(sub);
    return ORC_OK;
}

void orc_cdf_exclusive(const double *p, size_t n, double *cdf) {
    /* getCDFFunctor MeasuresFunctors.hpp:39-56 (exclusive scan) */
    double run = 0.0;
    for (size_t k = 0; k < n; k++) {
        const double v = p[k];
        cdf[k] = run;
        run += v;
    }
}

void orc_sample_from_uniforms(const double *cdf, size_t n, int nq,
                              const double *u, size_t shots, int64_t *out) {
    /* Sampler::operator() MeasuresFunctors.hpp:86-119 */
    for (size_t k = 0; k < shots; k++) {
        const double U = u[k];
        size_t index;
        if (U <= cdf[1]) {
            index = 0;
        } else {
            size_t lo = 1, hi = n, mid;
            double ct;
            while (hi - lo > 1) {
                mid = hi - ((hi - lo) >> 1);
                ct = (mid == n) ? 1.0 : cdf[mid];
                if (ct < U) lo = mid;
                else hi = mid;
            }
            index = hi - 1;
        }
        for (int j = 0; j < nq; j++) out[k * nq + (nq - 1 - j)] = (int64_t)((index >> j) & 1);
    }
}

/* ------------------------------------------------------------------------ */
/* adjoint Jacobian (AdjointDiffKokkos.hpp:404-478)                          */
/* ------------------------------------------------------------------------ */
int orc_adjoint_jacobian(const orc_cplx *lambda_in, int nq, orc_cplx *const *hl,
                         int nobs, int nops, const char *const *names,
                         const int64_t *wires, const int64_t *woff,
                         const double *params, const int64_t *poff,
                         const int32_t *inverses, const int64_t *tp, int ntp,
                         double *jac) {
    if (ntp <= 0) return ORC_BAD_ARGS; /* "No trainable parameters provided." */
    const size_t n = (size_t)1 << nq;
    orc_cplx *lam = (orc_cplx *)malloc(sizeof(orc_cplx) * n);
    orc_cplx *mu = (orc_cplx *)malloc(sizeof(orc_cplx) * n);
    if (!lam || !mu) {
        free(lam);
        free(mu);
        return ORC_BAD_ARGS;
    }
    memcpy(lam, lambda_in, sizeof(orc_cplx) * n);
    int num_param_ops = 0;
    for (int i = 0; i < nops; i++)
        if (poff[i + 1] > poff[i]) num_param_ops++;
    int tp_number = ntp - 1;
    long current_param_idx = num_param_ops - 1;
    int tp_it = ntp - 1; /* reverse iterator over trainable */
    int st = ORC_OK;
    for (int op = nops - 1; op >= 0; op--) {
        const int npar = (int)(poff[op + 1] - poff[op]);
        if (npar > 1) { st = ORC_BAD_ARGS; break; }
        if (strcmp(names[op], "StatePrep") == 0 || strcmp(names[op], "BasisState") == 0)
            continue;
        if (tp_it < 0) break;
        const int64_t *w = wires + woff[op];
        const int nw = (int)(woff[op + 1] - woff[op]);
        const double *p = params + poff[op];
        memcpy(mu, lam, sizeof(orc_cplx) * n);
        st = orc_apply(lam, nq, names[op], w, nw, !inverses[op], p, npar);
        if (st != ORC_OK) break;
        if (npar > 0) {
            if (current_param_idx == tp[tp_it]) {
                int gst;
                const double scale = orc_apply_generator(mu, nq, names[op], w, nw,
                                                         !inverses[op], &gst) *
                                     (inverses[op] ? -1.0 : 1.0);
                if (gst != ORC_OK) { st = gst; break; }
                for (int o = 0; o < nobs; o++)
                    jac[(size_t)o * ntp + tp_number] = -2.0 * scale * orc_inner_im(hl[o], mu, n);
                tp_number--;
                tp_it--;
            }
            current_param_idx--;
        }
        for (int o = 0; o < nobs; o++) {
            st = orc_apply(hl[o], nq, names[op], w, nw, !inverses[op], p, npar);
            if (st != ORC_OK) break;
        }
        if (st != ORC_OK) break;
    }
    free(lam);
    free(mu);
    return st;
}
