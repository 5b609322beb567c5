// ref_harness.cpp -- link-level driver around the reference program's own objects.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/ from the
// reference sources where they lie (never copied into this repository).  It runs,
// per channel, the same chain as Run_itrs (source/BcDor-Main.cpp:241-391) with
// Trel=7 ExtU1=1, one iteration:
//   Build_ExtendedHartreeFock + diag(xe) one-body term (:258, :275-341)
//   Build_Dynamic_SlfEn_2ndOrder                      (:347)
//   [Make_LancPivots + Reduce_SelfEn_Lncz]             (:371-374)
//   DysonMatrix                                       (:376 / :384)
// and writes every intermediate as FP64 into a tagged binary file, with the
// wall time of each of the three boundary calls (std::chrono), so the checker
// compares in-memory doubles rather than the 6-decimal text outputs.
//
// usage: bd_ref_harness <modspace> <propagator> <interaction> <pivots|-> <hw> <out.bin> [ish ...]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <vector>
using namespace std;

#include "BcDor-Global_variables.hh"
#include "BcDor-Run_vars.hh"

int DysonMatrix(Wide_self_energy_t *, SpProp_t *, double *, double *, double *);

static FILE *g_out = nullptr;

static void put(const char *tag, int kind, const void *data, long long count) {
    int len = (int)strlen(tag);
    fwrite(&len, 4, 1, g_out);
    fwrite(tag, 1, len, g_out);
    fwrite(&kind, 4, 1, g_out);
    fwrite(&count, 8, 1, g_out);
    if (count > 0) fwrite(data, kind == 0 ? 8 : 4, count, g_out);
}
static void putd(const char *tag, const double *d, long long n) { put(tag, 0, d, n); }
static void puti(const char *tag, const int *d, long long n) { put(tag, 1, d, n); }

int main(int argc, char **argv) {
    if (argc < 7) {
        fprintf(stderr, "usage: %s msp prop vpp pivots|- hw out.bin [ish...]\n", argv[0]);
        return 2;
    }
    BcDor_Init();
    Set_defaults();
    A = 16; Z = 8; N = 8;
    hwHO = atof(argv[5]);
    IU1body = 7; U1body_fac = 0.0;
    i_Ext_U1 = 1;
    i_2nd_ord = 1;
    const bool lanczos = strcmp(argv[4], "-") != 0;
    Lanczos = lanczos ? 2 : 0;
    if (lanczos) snprintf(DysPivots_file, 300, "%s", argv[4]);

    // quiet the reference's stdout chatter
    std::cout.setstate(std::ios_base::failbit);

    MS = new ModSpace_t(argv[1]);
    MS->Set_phys_const_hwHO(hwHO);
    auto t0 = chrono::steady_clock::now();
    Vpp = new VppInt_t(argv[3], MS);
    Vpp->check_for_double_entries();
    double t_load = chrono::duration<double>(chrono::steady_clock::now() - t0).count();
    SpProp_t *gin = new SpProp_t(argv[2], MS);

    g_out = fopen(argv[6], "wb");
    if (!g_out) return 3;

    vector<int> chans;
    for (int a = 7; a < argc; ++a) chans.push_back(atoi(argv[a]));
    if (chans.empty()) for (int s = 0; s < MS->nsubsh; ++s) chans.push_back(s);

    int NDIM = 0;
    for (int s = 0; s < MS->nsubsh; ++s) if (NDIM < MS->MSp_no[s]) NDIM = MS->MSp_no[s];
    int n_pvt_alloc = (10 > NDIM) ? 10 : NDIM;
    VectList Pivots(NDIM, n_pvt_alloc);
    Pivots.itype = Lanczos;

    // output propagator large enough for every solution
    long long cap = 30;
    {
        Wide_self_energy_t tmp(MS, Vpp, gin);
        for (int s = 0; s < MS->nsubsh; ++s) {
            int a1, a2;
            tmp.set_clj(s);
            tmp.Count_2p1h_2h1p_poles(&a1, &a2);
            cap += a1 + a2 + MS->MSp_no[s];
        }
    }
    SpProp_t *gout = new SpProp_t((int)cap, (int)cap, MS);

    double *Uab = new double[NDIM * NDIM];
    Wide_self_energy_t sfV, sfV_lncz;
    sfV.reset(MS, Vpp, gin);
    sfV_lncz.reset(MS, Vpp, gin);

    putd("t_load", &t_load, 1);
    for (int ish : chans) {
        char tg[64];
        sfV.set_clj(ish);
        sfV_lncz.set_clj(ish);
        sfV.Build_ExtendedHartreeFock();
        for (int i = 0; i < NDIM * NDIM; ++i) Uab[i] = 0.0;
        int nd = (NDIM < MS->MSp_no[ish]) ? NDIM : MS->MSp_no[ish];
        for (int i = 0; i < nd; ++i) Uab[i * (NDIM + 1)] = MS->MSp_xe[ish][i];
        sfV.Add_1bd_SelfEn(Uab, NDIM);
        const int D = sfV.NTOT_ORB;
        snprintf(tg, 64, "c%d/sig_hf", ish); putd(tg, sfV.Sig_HF, D * D);
        snprintf(tg, 64, "c%d/sig_1b", ish); putd(tg, sfV.Sig_1b, D * D);

        int n3, n4;
        auto ta = chrono::steady_clock::now();
        sfV.Build_Dynamic_SlfEn_2ndOrder(&n3, &n4, 1, 0, 0);
        auto tb = chrono::steady_clock::now();
        snprintf(tg, 64, "c%d/sig_fw", ish); putd(tg, sfV.Sig_dyn_fw, (long long)sfV.N_PLS_fw * sfV.NTOT_DIM);
        snprintf(tg, 64, "c%d/sig_bk", ish); putd(tg, sfV.Sig_dyn_bk, (long long)sfV.N_PLS_bk * sfV.NTOT_DIM);

        double x1 = 0, x2 = 0, x3 = 0;
        double t_lanczos = 0.0;
        chrono::steady_clock::time_point tc, td;
        if (lanczos) {
            Pivots.n_vcts = 0;
            Make_LancPivots(MS, &Pivots.n_vcts, Pivots.vect, Pivots.ia, Pivots.ib, ish, 0);
            tc = chrono::steady_clock::now();
            sfV_lncz.Reduce_SelfEn_Lncz(&sfV, Pivots.n_vcts, Pivots.vect, Pivots.ia, Pivots.ib, 1);
            td = chrono::steady_clock::now();
            t_lanczos = chrono::duration<double>(td - tc).count();
            snprintf(tg, 64, "c%d/sorted_fw", ish); putd(tg, sfV.Sig_dyn_fw, (long long)sfV.N_PLS_fw * sfV.NTOT_DIM);
            snprintf(tg, 64, "c%d/sorted_bk", ish); putd(tg, sfV.Sig_dyn_bk, (long long)sfV.N_PLS_bk * sfV.NTOT_DIM);
            snprintf(tg, 64, "c%d/lz_fw", ish); putd(tg, sfV_lncz.Sig_dyn_fw, (long long)sfV_lncz.N_PLS_fw * sfV_lncz.NTOT_DIM);
            snprintf(tg, 64, "c%d/lz_bk", ish); putd(tg, sfV_lncz.Sig_dyn_bk, (long long)sfV_lncz.N_PLS_bk * sfV_lncz.NTOT_DIM);
            int hdr[3] = {sfV_lncz.NTOT_DEN, sfV_lncz.n_piv_fw, sfV_lncz.n_piv_bk};
            snprintf(tg, 64, "c%d/lz_hdr", ish); puti(tg, hdr, 3);
            snprintf(tg, 64, "c%d/ipiv_fw", ish); puti(tg, sfV_lncz.i_piv_fw, sfV_lncz.NTOT_DIM);
            snprintf(tg, 64, "c%d/ipiv_bk", ish); puti(tg, sfV_lncz.i_piv_bk, sfV_lncz.NTOT_DIM);
            snprintf(tg, 64, "c%d/nitr", ish);
            vector<int> nit;
            for (int k = 0; k < Pivots.n_vcts; ++k) { nit.push_back(Pivots.ia[k]); nit.push_back(Pivots.ib[k]); }
            puti(tg, nit.data(), (long long)nit.size());
            tc = chrono::steady_clock::now();
            DysonMatrix(&sfV_lncz, gout, &x1, &x2, &x3);
            td = chrono::steady_clock::now();
        } else {
            tc = chrono::steady_clock::now();
            DysonMatrix(&sfV, gout, &x1, &x2, &x3);
            td = chrono::steady_clock::now();
        }
        double kol[3] = {x1, x2, x3};
        snprintf(tg, 64, "c%d/koltun", ish); putd(tg, kol, 3);
        double tm[3] = {chrono::duration<double>(tb - ta).count(), t_lanczos,
                        chrono::duration<double>(td - tc).count()};
        snprintf(tg, 64, "c%d/time", ish); putd(tg, tm, 3);
        // the solutions just appended to the output propagator (add_qp / add_qh layout)
        int np = gout->Sp_clj_np[ish], nh = gout->Sp_clj_nh[ish];
        vector<double> qp, qh;
        for (int k = 0; k < np; ++k) {
            qp.push_back(gout->Sp_clj_ep[ish][k]); qp.push_back(gout->Sp_clj_zp[ish][k]);
            for (int d = 0; d < D; ++d) qp.push_back(gout->Sp_clj_fqp[ish][k * gout->N_SPB_MX + d]);
        }
        for (int k = 0; k < nh; ++k) {
            qh.push_back(gout->Sp_clj_eh[ish][k]); qh.push_back(gout->Sp_clj_zh[ish][k]);
            for (int d = 0; d < D; ++d) qh.push_back(gout->Sp_clj_fqh[ish][k * gout->N_SPB_MX + d]);
        }
        snprintf(tg, 64, "c%d/qp", ish); putd(tg, qp.data(), (long long)qp.size());
        snprintf(tg, 64, "c%d/qh", ish); putd(tg, qh.data(), (long long)qh.size());
    }
    fclose(g_out);
    delete[] Uab;
    return 0;
}
