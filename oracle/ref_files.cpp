// ref_files.cpp -- link-level driver around the reference program's own objects that
// writes the reference's output files, for the golden file fixtures.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/ from the
// reference sources where they lie (never copied into this repository).  It loads a
// problem as Load_interaction / Run_itrs do (source/BcDor-Initialize.cpp:110-117,
// source/BcDor-Main.cpp:225) and writes, into <outdir>:
//   prop_written.dat     SpProp_t::write of the input propagator
//   pivots_written.dat   SpProp_t::DysPivots(.., n_bk = 3, n_fw = 5, z_cut = 60)
//   vpp_written.bin      VppInt_t::write (the .bin branch, write_bin)
//   vpp_list.bin         the loaded interaction list (tagged doubles / ints: iabJ, icdJ, V)
//   plain/, lanczos/     Wide_self_energy_t::save_SelfEn_bin of the listed channels, as the
//                        MakeSelfEn program saves them (source/BcDor-Miscellanea.cpp:176-267),
//                        without and with the Lanczos reduction, and their rows (sig.bin)
//
// usage: bd_ref_files <modspace> <propagator> <interaction> <pivots> <outdir> [ish ...]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>
using namespace std;

#include "BcDor-Global_variables.hh"
#include "BcDor-Run_vars.hh"

static FILE *g_out = nullptr;

static void put(const char *tag, int kind, const void *data, long long count) {
    int len = (int)strlen(tag);
    fwrite(&len, 4, 1, g_out);
    fwrite(tag, 1, len, g_out);
    fwrite(&kind, 4, 1, g_out);
    fwrite(&count, 8, 1, g_out);
    if (count > 0) fwrite(data, kind == 0 ? 8 : 4, count, g_out);
}

int main(int argc, char **argv) {
    if (argc < 6) {
        fprintf(stderr, "usage: %s msp prop vpp pivots outdir [ish...]\n", argv[0]);
        return 2;
    }
    BcDor_Init();
    Set_defaults();
    A = 16; Z = 8; N = 8;
    Lanczos = 2;
    snprintf(DysPivots_file, 300, "%s", argv[4]);
    std::cout.setstate(std::ios_base::failbit);
    const string out = argv[5];

    MS = new ModSpace_t(argv[1]);
    Vpp = new VppInt_t(argv[3], MS);
    Vpp->check_for_double_entries();
    SpProp_t *gin = new SpProp_t(argv[2], MS);

    gin->write((char *)(out + "/prop_written.dat").c_str());
    gin->DysPivots((char *)(out + "/pivots_written.dat").c_str(), 3, 5, 60.0);
    Vpp->write((char *)(out + "/vpp_written.bin").c_str());

    g_out = fopen((out + "/vpp_list.bin").c_str(), "wb");
    if (!g_out) return 3;
    int n = Vpp->n_me_stored;
    put("n", 1, &n, 1);
    put("iabJ", 1, Vpp->iabJ_list, n);
    put("icdJ", 1, Vpp->icdJ_list, n);
    put("V", 0, Vpp->Vpp_wrk, n);
    fclose(g_out);

    int NDIM = 0;
    for (int s = 0; s < MS->nsubsh; ++s) if (NDIM < MS->MSp_no[s]) NDIM = MS->MSp_no[s];
    VectList Pivots(NDIM, (10 > NDIM) ? 10 : NDIM);
    Pivots.itype = Lanczos;
    Wide_self_energy_t sfV(MS, Vpp, gin), sfV_lncz(MS, Vpp, gin);
    g_out = fopen((out + "/sig.bin").c_str(), "wb");
    if (!g_out) return 3;
    for (int a = 6; a < argc; ++a) {
        const int ish = atoi(argv[a]);
        char tg[64];
        int i1, i2;
        sfV.reset(ish, MS, Vpp, gin);
        sfV.Build_Dynamic_SlfEn_2ndOrder(&i1, &i2, 1, 0, 0);
        snprintf(sfV.STOREDIR, sizeof(sfV.STOREDIR), "%s/plain", out.c_str());
        sfV.save_SelfEn_bin(0);
        snprintf(tg, 64, "c%d/plain_fw", ish); put(tg, 0, sfV.Sig_dyn_fw, (long long)sfV.N_PLS_fw * sfV.NTOT_DIM);
        snprintf(tg, 64, "c%d/plain_bk", ish); put(tg, 0, sfV.Sig_dyn_bk, (long long)sfV.N_PLS_bk * sfV.NTOT_DIM);
        Pivots.n_vcts = 0;
        Make_LancPivots(MS, &Pivots.n_vcts, Pivots.vect, Pivots.ia, Pivots.ib, ish, 0);
        sfV_lncz.reset(ish, MS, Vpp, gin);
        sfV_lncz.Reduce_SelfEn_Lncz(&sfV, Pivots.n_vcts, Pivots.vect, Pivots.ia, Pivots.ib, 0);
        snprintf(sfV_lncz.STOREDIR, sizeof(sfV_lncz.STOREDIR), "%s/lanczos", out.c_str());
        sfV_lncz.save_SelfEn_bin(0);
        snprintf(tg, 64, "c%d/lz_fw", ish); put(tg, 0, sfV_lncz.Sig_dyn_fw, (long long)sfV_lncz.N_PLS_fw * sfV_lncz.NTOT_DIM);
        snprintf(tg, 64, "c%d/lz_bk", ish); put(tg, 0, sfV_lncz.Sig_dyn_bk, (long long)sfV_lncz.N_PLS_bk * sfV_lncz.NTOT_DIM);
        snprintf(tg, 64, "c%d/ipiv_fw", ish); put(tg, 1, sfV_lncz.i_piv_fw, sfV_lncz.NTOT_DIM);
        snprintf(tg, 64, "c%d/ipiv_bk", ish); put(tg, 1, sfV_lncz.i_piv_bk, sfV_lncz.NTOT_DIM);
        int hdr[2] = {sfV_lncz.NTOT_DEN, sfV.NTOT_DEN};
        snprintf(tg, 64, "c%d/nden", ish); put(tg, 1, hdr, 2);
    }
    fclose(g_out);
    return 0;
}
