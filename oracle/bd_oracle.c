/*
 * bd_oracle.c -- CPU restatement of the reference chain
 *   Sigma(2) build -> multi-pivot Lanczos reduction -> Dyson eigensolve
 * of BoccaDorata (craolus/BoccaDorata-public).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker used by tests/, by
 * __graft_entry__.smoke() and by bench.py's cpu_baseline / reference arm.  It is
 * never part of the product path (the product is the CUDA library under
 * boccadorata-public_gb300/).  Parity of this restatement is pinned against the
 * reference program itself, compiled from its own sources by oracle/Makefile
 * into oracle/_ref/, through the golden fixtures under tests/golden/.
 *
 * Every function states the reference lines it restates.  Floating-point
 * operations are written in the reference's order, and the file is compiled
 * with -ffp-contract=off so that no multiply-add is fused (the reference is
 * built for x86-64 without FMA).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <dlfcn.h>

#define SQR2 1.4142135623730950488016887
#define CHOFF (-2)
#define JMULT 128
#define ABMULT 1024
#define CHMULT 5

typedef struct {
    /* model space (per subshell) -- ModSpace_t, source/BcDor-Sp_classes.hh:32-79 */
    int nsubsh, norb, jmax, nspb;
    const int *l, *j2, *ip, *ch, *no, *orb_start;
    const int *orb_sh;
    /* propagator -- SpProp_t, source/BcDor-Sp_classes.hh:87-160 (fragment-major, stride nspb) */
    const int *np, *nh, *p_start, *h_start;
    const double *ep, *eh, *fqp, *fqh;
    int n_qp, n_qh;
    /* interaction, sorted canonical list -- VppInt_t, source/BcDor-Int_classes.hh:20-85 */
    int n_me;
    const int *iabJ, *icdJ;
    const double *V;
    const int *seg_str, *seg_end; /* Jipch_str / Jipch_end, CHMULT*JMULT*2 entries */
} bdo_problem;

/* ---------------------------------------------------------------------------
 * TriIneq (source/BcDor-Ang_momenta.hh:42-45): nonzero when the triangle
 * inequality fails.  Arguments are 2j values.
 * ------------------------------------------------------------------------- */
static int tri_fail(int a, int b, int c) {
    return (a + b < c) || (b + c < a) || (c + a < b);
}

static inline int ind_chipJ(int ch, int ip, int J) { return ((ch - CHOFF) * 2 + ip) * JMULT + J; }
static inline int ind_i1i2J(int i1, int i2, int J) { return (i1 * ABMULT + i2) * JMULT + J; }

/* ---------------------------------------------------------------------------
 * VppInt_t::prepare_for_reading's (ch,ip,J) segment table
 * (source/BcDor-Vpp_potential.cpp:440-501) for an already sorted list.
 * ------------------------------------------------------------------------- */
void bdo_segments(int n_me, const int *iabJ, const int *orb_sh, const int *sh_ch, const int *sh_ip,
                  int *seg_str, int *seg_end) {
    for (int i = 0; i < CHMULT * JMULT * 2; ++i) { seg_str[i] = -10; seg_end[i] = -10; }
    int prev = -1;
    for (int i = 0; i < n_me; ++i) {
        int k = iabJ[i], J = k % JMULT, ab = k / JMULT, a = ab / ABMULT, b = ab % ABMULT;
        int c = sh_ch[orb_sh[a]] + sh_ch[orb_sh[b]];
        int p = (sh_ip[orb_sh[a]] + sh_ip[orb_sh[b]]) % 2;
        int key = ind_chipJ(c, p, J);
        if (key != prev) {
            if (prev >= 0) seg_end[prev] = i - 1;
            seg_str[key] = i;
            prev = key;
        }
    }
    if (prev >= 0) seg_end[prev] = n_me - 1;
}

/* ---------------------------------------------------------------------------
 * VppInt_t::get (source/BcDor-Vpp_potential.cpp:557-607): canonicalise the
 * pairs with the exchange phase (-1)^((2ja+2jb)/2-J+1), order (ab)<=(cd),
 * then binary-search the (ch,ip,J) segment.  Missing elements are 0.
 * ------------------------------------------------------------------------- */
double bdo_vget(const bdo_problem *P, int ia, int ib, int ic, int id, int J) {
    int isha = P->orb_sh[ia], ishb = P->orb_sh[ib];
    int ip = (P->ip[isha] + P->ip[ishb]) % 2;
    int ch = P->ch[isha] + P->ch[ishb];
    int iph = 0, iab, icd;
    if (ia <= ib) iab = ind_i1i2J(ia, ib, J);
    else { iab = ind_i1i2J(ib, ia, J); iph += (P->j2[isha] + P->j2[ishb]) / 2 - J + 1; }
    if (ic <= id) icd = ind_i1i2J(ic, id, J);
    else {
        int ishc = P->orb_sh[ic], ishd = P->orb_sh[id];
        icd = ind_i1i2J(id, ic, J); iph += (P->j2[ishc] + P->j2[ishd]) / 2 - J + 1;
    }
    double xph = (double)(1 - 2 * (abs(iph) % 2));
    if (icd < iab) { int t = iab; iab = icd; icd = t; }
    int lo = P->seg_str[ind_chipJ(ch, ip, J)], hi = P->seg_end[ind_chipJ(ch, ip, J)];
    if (lo < 0 || hi < 0) return 0.0;
    for (int it = 0; it < 100; ++it) {
        int mid = (hi + lo) / 2;
        int am = P->iabJ[mid];
        int test = (iab < am);
        if (am == iab) {
            int cm = P->icdJ[mid];
            if (cm == icd) return P->V[mid] * xph;
            test = (icd < cm);
        }
        if (test) hi = mid;
        else { lo = mid; if (lo < hi) lo++; }
    }
    return 0.0;
}

/* ---------------------------------------------------------------------------
 * Wide_self_energy_t::Count_2p1h_2h1p_poles, all-poles branch
 * (source/BcDor-Self_energy_ext_Op_c.cpp:35-113).
 * ------------------------------------------------------------------------- */
void bdo_count_poles(const bdo_problem *P, int I, int *nfw, int *nbk) {
    *nfw = 0; *nbk = 0;
    for (int Jab = 0; Jab <= P->jmax; ++Jab)
        for (int ia = 0; ia < P->nsubsh; ++ia)
            for (int ib = ia; ib < P->nsubsh; ++ib) {
                if (tri_fail(P->j2[ia], P->j2[ib], 2 * Jab)) continue;
                int nJab = ((P->j2[ia] + P->j2[ib]) / 2 + Jab + 1) % 2;
                for (int ig = 0; ig < P->nsubsh; ++ig) {
                    if (P->ch[ia] + P->ch[ib] - P->ch[ig] != P->ch[I]) continue;
                    if ((P->ip[ia] + P->ip[ib] + P->ip[ig] + P->ip[I]) % 2 != 0) continue;
                    if (tri_fail(P->j2[ig], P->j2[I], 2 * Jab)) continue;
                    int na = P->np[ia], nb = P->np[ib], ng = P->nh[ig], s = na * nb * ng;
                    if (ia == ib) { nb = na + 1; if (nJab == 1) nb -= 2; s = (na * nb / 2) * ng; }
                    *nfw += s;
                    na = P->nh[ia]; nb = P->nh[ib]; ng = P->np[ig]; s = na * nb * ng;
                    if (ia == ib) { nb = na + 1; if (nJab == 1) nb -= 2; s = (na * nb / 2) * ng; }
                    *nbk += s;
                }
            }
}

/* ---------------------------------------------------------------------------
 * Wide_self_energy_t::Build_Dynamic_SlfEn_2ndOrder, all-poles branch
 * (source/BcDor-Self_energy_ext_Op_c.cpp:323-561).  Output rows of
 * NTOT_DIM = 2 + D doubles: [E, sum_d M_d^2, M_0 .. M_{D-1}], in the
 * reference's loop order Jab -> ia -> ib -> ig -> na -> nb -> ng.
 * Returns 0, or -1 if a capacity would be exceeded.
 * ------------------------------------------------------------------------- */
int bdo_sigma2(const bdo_problem *P, int I, double *sfw, int cap_fw, double *sbk, int cap_bk,
               int *nfw, int *nbk) {
    const int D = P->no[I], NDIM = 2 + D, NDEN = 2, NS = P->nspb;
    double *vbuf = (double *)malloc(sizeof(double) * (size_t)NS * NS * NS * NS + 8);
    int ifw = 0, ibk = 0;
    for (int Jab = 0; Jab <= P->jmax; ++Jab)
        for (int ia = 0; ia < P->nsubsh; ++ia)
            for (int ib = ia; ib < P->nsubsh; ++ib) {
                if (tri_fail(P->j2[ia], P->j2[ib], 2 * Jab)) continue;
                int nJab = abs((P->j2[ia] + P->j2[ib]) / 2 - Jab + 1) % 2;
                double xJab = (double)(1 - 2 * nJab);
                for (int ig = 0; ig < P->nsubsh; ++ig) {
                    int nJgd = abs((P->j2[ig] + P->j2[I]) / 2 - Jab + 1) % 2;
                    if (P->ch[ia] + P->ch[ib] - P->ch[ig] != P->ch[I]) continue;
                    if ((P->ip[ia] + P->ip[ib] + P->ip[ig] + P->ip[I]) % 2 != 0) continue;
                    if (tri_fail(P->j2[ig], P->j2[I], 2 * Jab)) continue;
                    /* V' gather, :396-421 */
                    double x3 = sqrt((double)(Jab + Jab + 1) / (double)(1 + P->j2[I]));
                    double *dv = vbuf;
                    for (int nd = 0; nd < P->no[I]; ++nd) {
                        int iid = P->orb_start[I] + nd;
                        for (int nas = 0; nas < P->no[ia]; ++nas) {
                            int nst = (ia == ib) ? nas + nJab : 0;
                            int iia = P->orb_start[ia] + nas;
                            for (int nbs = nst; nbs < P->no[ib]; ++nbs) {
                                int iib = P->orb_start[ib] + nbs;
                                for (int ngs = 0; ngs < P->no[ig]; ++ngs) {
                                    int iig = P->orb_start[ig] + ngs;
                                    if (iig == iid && nJgd) continue;
                                    *dv = x3 * bdo_vget(P, iia, iib, iid, iig, Jab);
                                    if (iig == iid) *dv *= SQR2;
                                    ++dv;
                                }
                            }
                        }
                    }
                    /* 2p1h (:425-481) then 2h1p (:484-539) */
                    for (int dir = 0; dir < 2; ++dir) {
                        const int *nA = dir == 0 ? P->np : P->nh, *nG = dir == 0 ? P->nh : P->np;
                        const int *sA = dir == 0 ? P->p_start : P->h_start, *sG = dir == 0 ? P->h_start : P->p_start;
                        const double *eA = dir == 0 ? P->ep : P->eh, *eG = dir == 0 ? P->eh : P->ep;
                        const double *fA = dir == 0 ? P->fqp : P->fqh, *fG = dir == 0 ? P->fqh : P->fqp;
                        double *out = dir == 0 ? sfw : sbk;
                        int *cnt = dir == 0 ? &ifw : &ibk;
                        int cap = dir == 0 ? cap_fw : cap_bk;
                        for (int na = 0; na < nA[ia]; ++na) {
                            int nst = (ia == ib) ? na + nJab : 0;
                            for (int nb = nst; nb < nA[ib]; ++nb)
                                for (int ng = 0; ng < nG[ig]; ++ng) {
                                    if (*cnt >= cap) { free(vbuf); return -1; }
                                    double *row = out + (size_t)(*cnt) * NDIM;
                                    const double *fa = fA + (size_t)(sA[ia] + na) * NS;
                                    const double *fb = fA + (size_t)(sA[ib] + nb) * NS;
                                    const double *fg = fG + (size_t)(sG[ig] + ng) * NS;
                                    row[0] = eA[sA[ia] + na] + eA[sA[ib] + nb] - eG[sG[ig] + ng];
                                    row[1] = 0.0;
                                    double x4 = 1.0;
                                    if (ia == ib && na == nb) x4 /= SQR2;
                                    dv = vbuf;
                                    for (int nd = 0; nd < P->no[I]; ++nd) {
                                        int iid = P->orb_start[I] + nd;
                                        double x1 = 0.0;
                                        for (int nas = 0; nas < P->no[ia]; ++nas) {
                                            int nst2 = (ia == ib) ? nas + nJab : 0;
                                            for (int nbs = nst2; nbs < P->no[ib]; ++nbs) {
                                                double x2 = fa[nas] * fb[nbs];
                                                if (ia == ib) {
                                                    x2 += xJab * fa[nbs] * fb[nas];
                                                    if (nas == nbs) x2 /= SQR2;
                                                }
                                                for (int ngs = 0; ngs < P->no[ig]; ++ngs) {
                                                    int iig = P->orb_start[ig] + ngs;
                                                    if (iig == iid && nJgd) continue;
                                                    x1 += (*dv) * x2 * fg[ngs];
                                                    ++dv;
                                                }
                                            }
                                        }
                                        x1 *= x4;
                                        row[NDEN + nd] = x1;
                                        row[1] += x1 * x1;
                                    }
                                    ++(*cnt);
                                }
                        }
                    }
                }
            }
    free(vbuf);
    *nfw = ifw; *nbk = ibk;
    return 0;
}

/* ---------------------------------------------------------------------------
 * Sort_u_double2dim / Sort_d_double2dim (source/BcDor-Utilities.cpp:25-94):
 * in-place heap sort of rows of ndim doubles by column isort, ascending (u)
 * or descending (d).  Deterministic; the order of equal keys is the heap's.
 * ------------------------------------------------------------------------- */
static void heap_rows(int ntot, int ndim, int isort, double *a, int desc) {
    if (ntot < 2) return;
    double *tmp = (double *)malloc(sizeof(double) * ndim);
    int l = ntot / 2, ir = ntot - 1, i, j;
    for (;;) {
        if (l > 0) {
            --l;
            memcpy(tmp, a + (size_t)l * ndim, sizeof(double) * ndim);
        } else {
            memcpy(tmp, a + (size_t)ir * ndim, sizeof(double) * ndim);
            memcpy(a + (size_t)ir * ndim, a, sizeof(double) * ndim);
            if (--ir == 0) { memcpy(a, tmp, sizeof(double) * ndim); break; }
        }
        i = l; j = l + l + 1;
        while (j <= ir) {
            double aj = a[(size_t)j * ndim + isort];
            if (j < ir) {
                double aj1 = a[(size_t)(j + 1) * ndim + isort];
                if (desc ? (aj > aj1) : (aj < aj1)) { j++; aj = aj1; }
            }
            if (desc ? (tmp[isort] > aj) : (tmp[isort] < aj)) {
                memcpy(a + (size_t)i * ndim, a + (size_t)j * ndim, sizeof(double) * ndim);
                i = j; j = j + j + 1;
            } else break;
        }
        memcpy(a + (size_t)i * ndim, tmp, sizeof(double) * ndim);
    }
    free(tmp);
}
void bdo_sort_u(int ntot, int ndim, int isort, double *a) { heap_rows(ntot, ndim, isort, a, 0); }
void bdo_sort_d(int ntot, int ndim, int isort, double *a) { heap_rows(ntot, ndim, isort, a, 1); }

/* Same heap sort, but only producing the row permutation from the key column
 * (used by tests to check the device's permutation of equal-energy rows). */
void bdo_sort_perm(int ntot, const double *key, int desc, int *perm) {
    double *rows = (double *)malloc(sizeof(double) * 2 * (ntot > 0 ? ntot : 1));
    for (int i = 0; i < ntot; ++i) { rows[2 * i] = key[i]; rows[2 * i + 1] = (double)i; }
    heap_rows(ntot, 2, 0, rows, desc);
    for (int i = 0; i < ntot; ++i) perm[i] = (int)rows[2 * i + 1];
    free(rows);
}

/* Deterministic pseudo-random restart value of pole i at Lanczos index j, in [0.5, 1.5)
 * (same function as the device's). */
static double restart_value(int i, int j) {
    unsigned x = (unsigned)i * 2654435761u ^ ((unsigned)j * 40503u + 0x9e3779b9u);
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return 0.5 + (double)(x & 0xffffffu) / 16777216.0;
}

/* ---------------------------------------------------------------------------
 * Reduce_Mtx_Lncz (source/BcDor-Lanczos.cpp:44-286).  Min rows are
 * [E, *, M_0..M_{NB_in-1}] (NA_in leading doubles); Mout rows are
 * [alpha, beta, g_0.., M'_0..] with NA_out leading doubles.  pivots is
 * nt_pvts rows of NB_in doubles and is normalised in place like the
 * reference.  Returns the number of Lanczos vectors, or < 0 on error.
 * ------------------------------------------------------------------------- */
int bdo_reduce_mtx_lncz_passes(int NA_out, int NB_out, int NPLS_out, double *Mout, int *i_piv_out,
                               int NA_in, int NB_in, int NPLS_in, const double *Min,
                               int nt_pvts, double *pivots, const int *n_itr, int passes) {
    if (NPLS_in < 1 || NPLS_out < 1) return -1;
    if (NB_out != NB_in) return -100;
    int nLanc = 0, jp = 0;
    for (int i = 0; i < nt_pvts; ++i) if (n_itr[i] > 0) { nLanc += n_itr[i]; ++jp; }
    if (nLanc < 1) return -2;
    if (nLanc > NPLS_in) nLanc = NPLS_in;
    if (nLanc > NPLS_out) return -100;
    if ((jp + 1 > NA_out) && (nLanc < NPLS_in)) return -100;
    const int NT_in = NA_in + NB_in, NT_out = NA_out + NB_out;
    int *i_last = (int *)malloc(sizeof(int) * (nt_pvts > 0 ? nt_pvts : 1));
    double *LV = (double *)malloc(sizeof(double) * (size_t)NPLS_in * nLanc);
    for (size_t q = 0; q < (size_t)NT_out * nLanc; ++q) Mout[q] = 0.0;
    double *re = Mout, *rm = Mout + NT_out - NB_out;
    for (int i = 0; i < nt_pvts; ++i) i_last[i] = -1000;
    int i_pvt = -1, n_pvt = -1, j_next = 0;
    for (int j = 0; j < nLanc; ++j) {
        double *vj = LV + (size_t)j * NPLS_in;
        int newv = (j == j_next);
        if (newv) {
            ++i_pvt;
            while (i_pvt < nt_pvts && n_itr[i_pvt] < 1) ++i_pvt;
            if (i_pvt >= nt_pvts) { free(i_last); free(LV); return -100; }
            ++n_pvt;
            j_next += n_itr[i_pvt];
            i_last[n_pvt] = j_next - 1;
            double *pv = pivots + (size_t)i_pvt * NB_in;
            double x1 = 0.0;
            for (int i = 0; i < NB_in; ++i) x1 += pv[i] * pv[i];
            x1 = sqrt(x1);
            for (int i = 0; i < NB_in; ++i) pv[i] /= x1;
            for (int k = 0; k < NPLS_in; ++k) {
                const double *ms = Min + (size_t)k * NT_in + NA_in;
                double s = 0.0;
                for (int l = 0; l < NB_in; ++l) s += ms[l] * pv[l];
                vj[k] = s;
            }
        } else {
            const double *vi = vj - NPLS_in;
            for (int k = 0; k < NPLS_in; ++k) vj[k] = vi[k] * Min[(size_t)k * NT_in];
        }
        double n0 = 0.0;
        for (int k = 0; k < NPLS_in; ++k) n0 += vj[k] * vj[k];
        /* backward modified Gram-Schmidt, :160-173 (passes > 1 repeats it) */
        for (int pass = 0; pass < passes; ++pass)
        for (int i = j - 1; i >= 0; --i) {
            const double *vi = LV + (size_t)i * NPLS_in;
            double x1 = 0.0, x2 = 0.0;
            for (int k = 0; k < NPLS_in; ++k) { x1 += vi[k] * vj[k]; x2 += vi[k] * vi[k]; }
            if (passes > 1 && x2 == 0.0) continue;   /* multi-sweep mode skips empty vectors */
            for (int k = 0; k < NPLS_in; ++k) vj[k] -= x1 * vi[k] / x2;
        }
        int injected = 0;
        if (passes > 1) {
            /* Exhausted reachable subspace (not part of the reference, whose rows become
             * NaN here): continue with the unit vector of the first pole no stored vector
             * touches (alpha = E_k, beta = 0, g = 0, m = M[k, :]), else with a
             * pseudo-random vector swept orthogonal to the basis (beta = 0). */
            double nn = 0.0;
            for (int k = 0; k < NPLS_in; ++k) nn += vj[k] * vj[k];
            if (nn <= 1e-48 * n0 || nn == 0.0) {
                int kfree = -1;
                for (int k = 0; k < NPLS_in && kfree < 0; ++k) {
                    int used = 0;
                    for (int i = 0; i < j && !used; ++i) used = (LV[(size_t)i * NPLS_in + k] != 0.0);
                    if (!used) kfree = k;
                }
                if (kfree >= 0) {
                    for (int k = 0; k < NPLS_in; ++k) vj[k] = (k == kfree) ? 1.0 : 0.0;
                    re[0] = Min[(size_t)kfree * NT_in];
                    for (int l = 0; l < NB_out; ++l) rm[l] = Min[(size_t)kfree * NT_in + NA_in + l];
                    rm += NT_out; re += NT_out;
                    continue;
                }
                for (int k = 0; k < NPLS_in; ++k) vj[k] = restart_value(k, j);
                for (int pass = 0; pass < passes; ++pass)
                    for (int i = j - 1; i >= 0; --i) {
                        const double *vi = LV + (size_t)i * NPLS_in;
                        double x1 = 0.0, x2 = 0.0;
                        for (int k = 0; k < NPLS_in; ++k) { x1 += vi[k] * vj[k]; x2 += vi[k] * vi[k]; }
                        if (x2 > 0.0) for (int k = 0; k < NPLS_in; ++k) vj[k] -= x1 * vi[k] / x2;
                    }
                injected = 1;
            }
        }
        /* alpha, beta, coupling, :180-216 */
        double xa = 0.0, xb = 0.0;
        for (int k = 0; k < NPLS_in; ++k) {
            double x1 = vj[k];
            const double *ms = Min + (size_t)k * NT_in;
            xa += ms[0] * x1 * x1;
            xb += x1 * x1;
            for (int l = 0; l < NB_out; ++l) rm[l] += ms[NA_in + l] * x1;
        }
        xa /= xb;
        xb = sqrt(xb);
        re[0] = xa;
        re[1] = xb;
        for (int l = 0; l < NB_out; ++l) rm[l] /= xb;
        for (int i = 0; i < n_pvt; ++i) {
            const double *vi = LV + (size_t)i_last[i] * NPLS_in;
            double xg = 0.0;
            for (int k = 0; k < NPLS_in; ++k) xg += Min[(size_t)k * NT_in] * vi[k] * vj[k];
            re[2 + i] = xg / xb;
        }
        for (int k = 0; k < NPLS_in; ++k) vj[k] /= xb;
        if (injected) re[1] = 0.0;
        if (newv) re[1] = re[1 + n_pvt];
        if (n_pvt + 2 + NB_out > NT_out) { free(i_last); free(LV); return -200; }
        rm += NT_out; re += NT_out;
    }
    ++n_pvt;
    i_piv_out[0] = n_pvt;
    i_piv_out[1] = 1;
    for (int i = 0; i < n_pvt; ++i) i_piv_out[2 + i] = i_last[i] + 1;
    int ok = (i_last[n_pvt - 1] + 1 == nLanc) || ((i_last[n_pvt - 1] + 1 > nLanc) && (NPLS_in == nLanc));
    free(i_last); free(LV);
    return ok ? nLanc : -200;
}

/* The reference's single-pass form, bit-identical to Reduce_Mtx_Lncz. */
int bdo_reduce_mtx_lncz(int NA_out, int NB_out, int NPLS_out, double *Mout, int *i_piv_out,
                        int NA_in, int NB_in, int NPLS_in, const double *Min,
                        int nt_pvts, double *pivots, const int *n_itr) {
    return bdo_reduce_mtx_lncz_passes(NA_out, NB_out, NPLS_out, Mout, i_piv_out, NA_in, NB_in, NPLS_in, Min,
                                      nt_pvts, pivots, n_itr, 1);
}

/* ---------------------------------------------------------------------------
 * Sizes of Reduce_SelfEn_Lncz (source/BcDor-Self_energy_ext_Op_e.cpp:161-203):
 * nLanc = min(sum of positive n_itr, N); when the sum exceeds N the iteration
 * counts are rescaled in place to int(N/sum*n_itr + 1).
 * ------------------------------------------------------------------------- */
int bdo_lanczos_sizes(int nt_pvts, int *n_itr, int N) {
    int tot = 0;
    for (int i = 0; i < nt_pvts; ++i) if (n_itr[i] > 0) tot += n_itr[i];
    int nL = tot < N ? tot : N;
    if (N < 1 || nL < 1) return nL < 0 ? 0 : nL;
    if (tot > N) {
        double x1 = (double)N / (double)tot;
        for (int i = 0; i < nt_pvts; ++i) n_itr[i] = (int)(x1 * n_itr[i] + 1.0);
    }
    return nL;
}

/* ---------------------------------------------------------------------------
 * SpProp_t::ExtendedHartreeFock_Pot (source/BcDor-Sp_Propagator_a.cpp:39-130)
 * for channel I into U[D*D].
 * ------------------------------------------------------------------------- */
void bdo_ehf(const bdo_problem *P, int I, double *U) {
    const int D = P->no[I], NS = P->nspb;
    for (int nc = 0; nc < D; nc++)
        for (int nr = nc; nr < D; nr++) {
            double U_ehf = 0.0;
            for (int iv = 0; iv < P->nsubsh; ++iv) {
                int J2l = abs(P->j2[I] - P->j2[iv]), J2u = P->j2[I] + P->j2[iv];
                for (int J2 = J2l; J2 <= J2u; J2 += 2) {
                    int nJ = ((P->j2[I] + P->j2[iv] + J2) / 2) % 2;
                    double x1 = (double)(J2 + 1) / (double)(P->j2[I] + 1);
                    double x7 = 0.0;
                    for (int nm = 0; nm < P->no[iv]; nm++) {
                        if (iv == I && nm == nr && nJ != 1) continue;
                        double x2 = (iv == I && nm == nr) ? SQR2 : 1.0;
                        int ia = P->orb_start[I] + nr, im = P->orb_start[iv] + nm;
                        for (int nv = 0; nv < P->no[iv]; nv++) {
                            if (iv == I && nv == nc && nJ != 1) continue;
                            double x3 = (iv == I && nv == nc) ? SQR2 : 1.0;
                            int ib = P->orb_start[I] + nc, iu = P->orb_start[iv] + nv;
                            double x6 = 0.0;
                            const double *q = P->fqh + (size_t)P->h_start[iv] * NS;
                            for (int kg = 0; kg < P->nh[iv]; ++kg) { x6 += q[nv] * q[nm]; q += NS; }
                            x7 = x7 + x2 * x3 * x6 * bdo_vget(P, ia, im, ib, iu, J2 / 2);
                        }
                    }
                    U_ehf = U_ehf + x1 * x7;
                }
            }
            U[nr * D + nc] = U_ehf;
            U[nc * D + nr] = U_ehf;
        }
}

/* ---------------------------------------------------------------------------
 * Seek_EFermi (source/BcDor-DysonMatrix.cpp:619-635) on the input propagator.
 * ------------------------------------------------------------------------- */
double bdo_seek_efermi(const bdo_problem *P, int I) {
    int ch = P->ch[I];
    double x1 = P->ep[0] + 100., x2 = P->eh[0] - 100.;
    for (int s = 0; s < P->nsubsh; ++s) {
        if (P->ch[s] != ch) continue;
        for (int k = 0; k < P->np[s]; ++k) if (P->ep[P->p_start[s] + k] < x1) x1 = P->ep[P->p_start[s] + k];
        for (int k = 0; k < P->nh[s]; ++k) if (P->eh[P->h_start[s] + k] > x2) x2 = P->eh[P->h_start[s] + k];
    }
    return (x1 + x2) / 2.0;
}

/* ---------------------------------------------------------------------------
 * Symmetric eigensolver used by the Dyson step.  The reference calls LAPACK
 * dsyevd_("V","U") (source/BcDor-DysonMatrix.cpp:35-36,412).  When a LAPACK
 * library has been registered with bdo_set_lapack(), its dsyevd_ is called the
 * same way; otherwise a Householder tridiagonalisation (lower variant,
 * written out below) followed by the implicit QL iteration of EISPACK's
 * public-domain tql2 is used.
 * ------------------------------------------------------------------------- */
typedef void (*dsyevd_fn)(char *, char *, int *, double *, int *, double *, double *, int *, int *, int *, int *);
static dsyevd_fn g_dsyevd = NULL;

int bdo_set_lapack(const char *path, const char *symbol) {
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    g_dsyevd = (dsyevd_fn)dlsym(h, symbol);
    return g_dsyevd ? 0 : -2;
}
int bdo_has_lapack(void) { return g_dsyevd != NULL; }

/* a: n x n, column j of eigenvectors in a[j*lda .. ] on exit (LAPACK layout),
 * w ascending. */
static int sym_eig(int n, double *a, int lda, double *w) {
    if (n < 1) return 0;
    if (g_dsyevd) {
        int lwork = 2 + (6 + 2 * n) * n, liwork = 3 + 5 * n, info = 0;
        double *work = (double *)malloc(sizeof(double) * lwork);
        int *iwork = (int *)malloc(sizeof(int) * liwork);
        char jobz = 'V', uplo = 'U';
        g_dsyevd(&jobz, &uplo, &n, a, &lda, w, work, &lwork, iwork, &liwork, &info);
        free(work); free(iwork);
        return info;
    }
    /* Householder reduction A = Q T Q^T, lower variant: step k builds the
     * reflector H_k = I - tau v v^T (v[0..k] = 0, v[k+1] = 1) that zeroes
     * A[k+2.., k]; p = tau A v, w = p - (tau/2)(p.v) v, A -= v w^T + w v^T. */
    double *z = (double *)malloc(sizeof(double) * (size_t)n * n), *e = (double *)calloc(n, sizeof(double));
    double *A = (double *)malloc(sizeof(double) * (size_t)n * n), *vs = (double *)calloc((size_t)n * n, sizeof(double));
    double *taus = (double *)calloc(n, sizeof(double)), *pw = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) A[(size_t)i * n + j] = a[(size_t)j * lda + i];
    for (int k = 0; k + 2 < n; ++k) {
        double alpha = A[(size_t)(k + 1) * n + k], sig = 0.0;
        for (int i = k + 2; i < n; ++i) sig += A[(size_t)i * n + k] * A[(size_t)i * n + k];
        double *v = vs + (size_t)k * n;
        if (sig == 0.0) { taus[k] = 0.0; e[k] = alpha; continue; }
        double beta = -copysign(sqrt(alpha * alpha + sig), alpha);
        double tau = (beta - alpha) / beta, scal = 1.0 / (alpha - beta);
        v[k + 1] = 1.0;
        for (int i = k + 2; i < n; ++i) v[i] = A[(size_t)i * n + k] * scal;
        taus[k] = tau; e[k] = beta;
        double pv = 0.0;
        for (int i = k + 1; i < n; ++i) {
            double s = 0.0;
            for (int j = k + 1; j < n; ++j) s += A[(size_t)i * n + j] * v[j];
            pw[i] = tau * s; pv += pw[i] * v[i];
        }
        for (int i = k + 1; i < n; ++i) pw[i] -= 0.5 * tau * pv * v[i];
        for (int i = k + 1; i < n; ++i)
            for (int j = k + 1; j < n; ++j) A[(size_t)i * n + j] -= v[i] * pw[j] + pw[i] * v[j];
    }
    for (int i = 0; i < n; ++i) w[i] = A[(size_t)i * n + i];
    if (n >= 2) e[n - 2] = A[(size_t)(n - 1) * n + (n - 2)];
    /* Q = H_0 H_1 ... accumulated backwards into z (row-major, column = vector) */
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) z[(size_t)i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int k = n - 3; k >= 0; --k) {
        const double *v = vs + (size_t)k * n;
        if (taus[k] == 0.0) continue;
        for (int j = k + 1; j < n; ++j) {
            double s = 0.0;
            for (int i = k + 1; i < n; ++i) s += v[i] * z[(size_t)i * n + j];
            s *= taus[k];
            for (int i = k + 1; i < n; ++i) z[(size_t)i * n + j] -= s * v[i];
        }
    }
    free(A); free(vs); free(taus); free(pw);
    /* e[i] couples rows i and i+1; the QL loop below expects that layout */
    /* implicit QL with shifts (EISPACK tql2, public domain) */
    e[n - 1] = 0.0;
    double f = 0.0, tst1 = 0.0;
    for (int l = 0; l < n; ++l) {
        double hh = fabs(w[l]) + fabs(e[l]);
        if (tst1 < hh) tst1 = hh;
        int m = l;
        while (m < n - 1 && fabs(e[m]) > 2.220446049250313e-16 * tst1) ++m;
        if (m > l) {
            int iter = 0;
            do {
                if (++iter > 200) { free(z); free(e); return 1; }
                double g = w[l], p = (w[l + 1] - g) / (2.0 * e[l]), r = hypot(p, 1.0);
                if (p < 0) r = -r;
                w[l] = e[l] / (p + r); w[l + 1] = e[l] * (p + r);
                double dl1 = w[l + 1], h = g - w[l];
                for (int i = l + 2; i < n; ++i) w[i] -= h;
                f += h;
                p = w[m];
                double c = 1.0, c2 = 1.0, c3 = 1.0, el1 = e[l + 1], s = 0.0, s2 = 0.0;
                for (int i = m - 1; i >= l; --i) {
                    c3 = c2; c2 = c; s2 = s;
                    g = c * e[i]; h = c * p; r = hypot(p, e[i]);
                    e[i + 1] = s * r; s = e[i] / r; c = p / r;
                    p = c * w[i] - s * g;
                    w[i + 1] = h + s * (c * g + s * w[i]);
                    for (int k = 0; k < n; ++k) {
                        h = z[(size_t)k * n + i + 1];
                        z[(size_t)k * n + i + 1] = s * z[(size_t)k * n + i] + c * h;
                        z[(size_t)k * n + i] = c * z[(size_t)k * n + i] - s * h;
                    }
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p; w[l] = c * p;
            } while (fabs(e[l]) > 2.220446049250313e-16 * tst1);
        }
        w[l] = w[l] + f; e[l] = 0.0;
    }
    /* ascending order with vectors */
    for (int i = 0; i < n - 1; ++i) {
        int k = i; double p = w[i];
        for (int j = i + 1; j < n; ++j) if (w[j] < p) { k = j; p = w[j]; }
        if (k != i) {
            w[k] = w[i]; w[i] = p;
            for (int j = 0; j < n; ++j) { double t = z[(size_t)j * n + i]; z[(size_t)j * n + i] = z[(size_t)j * n + k]; z[(size_t)j * n + k] = t; }
        }
    }
    for (int j = 0; j < n; ++j) for (int i = 0; i < n; ++i) a[(size_t)j * lda + i] = z[(size_t)i * n + j];
    free(z); free(e);
    return 0;
}

/* ---------------------------------------------------------------------------
 * Calc_En (source/BcDor-DysonMatrix.cpp:542-594): Koltun partial sums over
 * the quasihole rows (sorted descending), three magnitude buckets.
 * ------------------------------------------------------------------------- */
static void calc_en(int D, const double *sig1b, int j2, int nsolb, int NDIM, const double *solb,
                    double *e1b, double *esum, double *asum) {
    double a1 = 0, a2 = 0, a3 = 0, b1 = 0, b2 = 0, b3 = 0, c1 = 0, c2 = 0, c3 = 0;
    for (int ne = nsolb - 1; ne >= 0; --ne) {
        const double *p1 = solb + (size_t)ne * NDIM, *p2 = p1 + 2;
        double x1 = 0.0, x2 = 0.0;
        for (int nr = 0; nr < D; ++nr) {
            x1 += p2[nr] * p2[nr];
            for (int nc = 0; nc < D; ++nc) x2 += sig1b[nr * D + nc] * p2[nr] * p2[nc];
        }
        if (x1 > 0.01) { a1 += x2; b1 += x1 * p1[0]; c1 += x1; }
        else if (x1 > 1.e-5) { a2 += x2; b2 += x1 * p1[0]; c2 += x1; }
        else { a3 += x2; b3 += x1 * p1[0]; c3 += x1; }
    }
    double x = (double)j2 + 1.0;
    *e1b = (a1 + a2 + a3) * x; *esum = (b1 + b2 + b3) * x; *asum = (c1 + c2 + c3) * x;
}

/* ---------------------------------------------------------------------------
 * DysonMatrix (source/BcDor-DysonMatrix.cpp:123-532) without the HFB branch.
 * sig1b, sighf: D x D.  fw/bk: self-energy rows of NDIM_se = NDEN + D doubles
 * (NDEN = 2 for a plain Sigma(2), n_pvt+1 after Lanczos).  n_piv_* = 0 means
 * "not Lanczos-reduced": the rows are then sorted in place like the reference
 * (fw descending, bk ascending).  ipiv_*: i_piv arrays (may be NULL when
 * n_piv_* == 0).  Outputs: sol (n x (2+D) rows: first nsolf qp rows sorted
 * descending, then nsolb qh rows sorted descending), koltun[3].
 * Returns 0 or the LAPACK info.
 * ------------------------------------------------------------------------- */
int bdo_dyson(int D, int j2, const double *sig1b, const double *sighf, double efermi,
              int NDEN, int nfw, double *fw, int n_piv_fw, const int *ipiv_fw,
              int nbk, double *bk, int n_piv_bk, const int *ipiv_bk,
              double *sol, int *nsolf_out, int *nsolb_out, double *koltun) {
    const int NDIM_se = NDEN + D, NSOL = D + 2;
    if (n_piv_fw == 0 && nfw > 0) bdo_sort_d(nfw, NDIM_se, 0, fw);
    if (n_piv_bk == 0 && nbk > 0) bdo_sort_u(nbk, NDIM_se, 0, bk);
    int n = D + (nfw > 0 ? nfw : 0) + (nbk > 0 ? nbk : 0), LDA = n + 1;
    double *A = (double *)calloc((size_t)LDA * LDA, sizeof(double));
    double *W = (double *)malloc(sizeof(double) * LDA);
    for (int r = 0; r < D; ++r) for (int c = 0; c < D; ++c) A[(size_t)r * LDA + c] = sig1b[r * D + c] + sighf[r * D + c];
    for (int part = 0; part < 2; ++part) {
        int np = part == 0 ? nfw : nbk, off = D + (part == 0 ? 0 : nfw), npiv = part == 0 ? n_piv_fw : n_piv_bk;
        const double *rows = part == 0 ? fw : bk;
        const int *ipiv = part == 0 ? ipiv_fw : ipiv_bk;
        if (np <= 0) continue;
        for (int i = 0; i < np; ++i) {
            const double *row = rows + (size_t)i * NDIM_se;
            A[(size_t)(off + i) * LDA + off + i] = row[0];
            for (int r = 0; r < D; ++r) {
                A[(size_t)(off + i) * LDA + r] = row[NDEN + r];
                A[(size_t)r * LDA + off + i] = row[NDEN + r];
            }
        }
        if (npiv > 0) {
            /* tridiagonal beta plus the fishbone branches, :303-333 / :359-389 */
            int nc = 1;
            for (int i = 1; i < np; ++i) {
                const double *row = rows + (size_t)i * NDIM_se;
                A[(size_t)(off + i - 1) * LDA + off + i] = row[1];
                A[(size_t)(off + i) * LDA + off + i - 1] = row[1];
                if (i == ipiv[nc + 1]) {
                    for (int nr = i; nr < np; ++nr) {
                        double g = rows[(size_t)nr * NDIM_se + 1 + nc];
                        A[(size_t)(off + i - 1) * LDA + off + nr] = g;
                        A[(size_t)(off + nr) * LDA + off + i - 1] = g;
                    }
                    ++nc;
                }
            }
            if (nc > npiv) { free(A); free(W); return -300; }
        }
    }
    int info = sym_eig(n, A, LDA, W);
    if (info != 0) { free(A); free(W); return info; }
    double *solf = sol, *solb = sol + (size_t)n * NSOL;
    int nsolf = 0, nsolb = 0;
    for (int ne = 0; ne < n; ++ne) {
        const double *v = A + (size_t)ne * LDA;
        double x1 = 0, x2 = 0;
        for (int i = 0; i < n; ++i) { x1 += v[i] * v[i]; if (i < D) x2 += v[i] * v[i]; }
        double *dst;
        if (W[ne] > efermi) { dst = solf; solf += NSOL; ++nsolf; }
        else { solb -= NSOL; ++nsolb; dst = solb; }
        dst[0] = W[ne]; dst[1] = x2 / x1;
        for (int i = 0; i < D; ++i) dst[2 + i] = v[i];
    }
    bdo_sort_d(nsolf, NSOL, 0, sol);
    bdo_sort_d(nsolb, NSOL, 0, sol + (size_t)nsolf * NSOL);
    /* add_qp / add_qh recompute Z as sum of squared amplitudes (source/BcDor-Sp_Propagator.cpp:726-734) */
    for (int k = 0; k < n; ++k) {
        double *r = sol + (size_t)k * NSOL, z = 0.0;
        for (int i = 0; i < D; ++i) z += r[2 + i] * r[2 + i];
        r[1] = z;
    }
    calc_en(D, sig1b, j2, nsolb, NSOL, sol + (size_t)nsolf * NSOL, &koltun[0], &koltun[1], &koltun[2]);
    *nsolf_out = nsolf; *nsolb_out = nsolb;
    free(A); free(W);
    return 0;
}
