// bd_files.cu -- the reference's input and output files: model space, propagator,
// Lanczos pivots, interaction (.bcd text and .bin), and the self-energy's binary form.
//
// Readers follow the reference's own (each function cites the one it restates) and
// keep what it keeps; nothing here exits the process: a malformed file gives a status
// code and a message (bd_files_error).  The interaction's lines are kept as read
// (orbits, J, V in file order); bd_upload_files puts them in the canonical order on
// the device (k_vpp_canon, the radix sort of k_sort.cu, k_vpp_place) instead of the
// reference's host heap sort, which takes 44 % of its run at N_max = 10.
#include <algorithm>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/bd_gb300.h"
#include "bd_common.cuh"
#include "bd_kernels.h"

using bd::kABMult;
using bd::kJMult;

struct bd_files {
    std::string err;
    // model space (ModSpace_t)
    int nsubsh = 0, norb = 0;
    std::vector<int> l, j2, ip, ch, no, nqp, nqh, orb_sh, orb_n, orb_F, orb_start;
    std::vector<double> orb_xe;
    std::vector<std::string> names;
    std::vector<const char *> name_ptr;
    // propagator (SpProp_t)
    bool have_prop = false;
    int nspb = 0;
    std::vector<int> np, nh;
    std::vector<double> ep, eh, zp, zh, fqp, fqh;
    // pivots (Make_LancPivots, every subshell)
    bool have_piv = false;
    std::vector<int> npvt, nfw, nbk;
    std::vector<double> pvec;
    // interaction lines kept, in file order: orbits a, b, c, d, J and V
    bool have_vpp = false;
    std::vector<int4> vabcd;
    std::vector<int> vJ;
    std::vector<double> vV;
    long long n_outside = 0, n_pauli = 0, n_alloc = 0;
};

namespace {

int ffail(bd_files *f, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (f) f->err = buf;
    return code;
}

// The whole file in memory, and its lines as fgets gives them (without the newline).
struct TextFile {
    std::string data;
    std::vector<size_t> start;   // line starts
    bool load(const char *path) {
        FILE *fp = std::fopen(path, "rb");
        if (!fp) return false;
        std::fseek(fp, 0, SEEK_END);
        const long sz = std::ftell(fp);
        std::fseek(fp, 0, SEEK_SET);
        data.resize(sz > 0 ? (size_t)sz : 0);
        const size_t got = sz > 0 ? std::fread(&data[0], 1, (size_t)sz, fp) : 0;
        std::fclose(fp);
        if (got != data.size()) return false;
        return true;
    }
    void index(size_t from = 0, size_t max_lines = (size_t)-1) {
        start.clear();
        size_t p = from;
        while (p < data.size() && start.size() < max_lines) {
            start.push_back(p);
            const void *nl = std::memchr(data.data() + p, '\n', data.size() - p);
            if (!nl) break;
            p = (size_t)(static_cast<const char *>(nl) - data.data()) + 1;
        }
    }
    std::string line(size_t k) const {
        if (k >= start.size()) return std::string();
        const size_t a = start[k];
        size_t b = data.find('\n', a);
        if (b == std::string::npos) b = data.size();
        return data.substr(a, b - a);
    }
};

// sscanf-like scanners over one line: "%i" (strtol base 0) and "%lf" (strtod), each
// skipping leading white space; they return false where sscanf would stop.
bool scan_int(const char *&p, int &v) {
    char *e = nullptr;
    errno = 0;
    const long x = std::strtol(p, &e, 0);
    if (e == p) return false;
    v = (int)x;
    p = e;
    return true;
}
bool scan_dbl(const char *&p, double &v) {
    char *e = nullptr;
    const double x = std::strtod(p, &e);
    if (e == p) return false;
    v = x;
    p = e;
    return true;
}
// the literal text of a format: white space matches any white space, '#' and letters themselves
bool scan_lit(const char *&p, const char *lit) {
    for (const char *q = lit; *q; ++q) {
        if (*q == ' ') {
            while (*p == ' ' || *p == '\t' || *p == '\r') ++p;
            continue;
        }
        if (*p != *q) return false;
        ++p;
    }
    return true;
}

}  // namespace

extern "C" {

const char *bd_files_error(const bd_files *f) { return f ? f->err.c_str() : "null files object"; }

void bd_files_close(bd_files *f) { delete f; }

// ModSpace_t::ModSpace_t(char*) (source/BcDor-Mod_Space.cpp:415-505).
int bd_files_open(bd_files **out, const char *path) {
    if (!out || !path) return BD_ERR_ARG;
    *out = nullptr;
    bd_files *f = new bd_files();
    TextFile t;
    if (!t.load(path)) {
        *out = f;
        return ffail(f, BD_ERR_ARG, "model space '%s': cannot read the file", path);
    }
    t.index();
    size_t k = 4;   // two header lines, a blank line, the "# number of" line
    int ns = 0, no_tot = 0;
    {
        const std::string s = t.line(k++);
        const char *p = s.c_str();
        if (!scan_int(p, ns) || !scan_int(p, no_tot) || ns < 1 || no_tot < 1) {
            *out = f;
            return ffail(f, BD_ERR_ARG, "model space '%s': no subshell / orbit counts on line 5", path);
        }
    }
    f->nsubsh = ns;
    f->norb = no_tot;
    int orb = 0;
    for (int i = 0; i < ns; ++i) {
        ++k;   // blank line
        std::string s = t.line(k++);
        const char *p = s.c_str();
        char name[16] = {0};
        if (!scan_lit(p, "# subshell: ")) { *out = f; return ffail(f, BD_ERR_ARG, "model space '%s': subshell %d header", path, i); }
        while (*p == ' ') ++p;
        int nn = 0;
        while (*p && *p != ' ' && *p != '\t' && *p != '\r' && nn < 8) name[nn++] = *p++;
        f->names.push_back(name);
        int a[4], b[3];
        s = t.line(k++);
        p = s.c_str();
        for (int q = 0; q < 4; ++q)
            if (!scan_int(p, a[q])) { *out = f; return ffail(f, BD_ERR_ARG, "model space '%s': quantum numbers of subshell %d", path, i); }
        s = t.line(k++);
        p = s.c_str();
        for (int q = 0; q < 3; ++q)
            if (!scan_int(p, b[q])) { *out = f; return ffail(f, BD_ERR_ARG, "model space '%s': orbit counts of subshell %d", path, i); }
        f->l.push_back(a[0]); f->j2.push_back(a[1]); f->ip.push_back(a[2]); f->ch.push_back(a[3]);
        f->no.push_back(b[0]); f->nqp.push_back(b[1]); f->nqh.push_back(b[2]);
        f->orb_start.push_back(orb);
        ++k;   // "# principal q.#" line
        for (int j = 0; j < b[0]; ++j) {
            s = t.line(k++);
            p = s.c_str();
            int n1, n2;
            double x;
            if (!scan_int(p, n1) || !scan_int(p, n2) || !scan_dbl(p, x))
                { *out = f; return ffail(f, BD_ERR_ARG, "model space '%s': orbit %d of subshell %d", path, j, i); }
            f->orb_sh.push_back(i); f->orb_n.push_back(n1); f->orb_F.push_back(n2); f->orb_xe.push_back(x);
            ++orb;
        }
    }
    if (orb != no_tot) { *out = f; return ffail(f, BD_ERR_ARG, "model space '%s': %d orbits listed, %d declared", path, orb, no_tot); }
    for (auto &n : f->names) f->name_ptr.push_back(n.c_str());
    *out = f;
    return BD_OK;
}

int bd_files_modspace(const bd_files *f, bd_modspace *ms, const int **orb_n, const char *const **names) {
    if (!f || !ms || f->nsubsh < 1) return BD_ERR_STATE;
    ms->nsubsh = f->nsubsh;
    ms->norb = f->norb;
    ms->l = f->l.data(); ms->j2 = f->j2.data(); ms->ip = f->ip.data(); ms->ch = f->ch.data(); ms->no = f->no.data();
    ms->orb_sh = f->orb_sh.data();
    ms->orb_xe = f->orb_xe.data();
    if (orb_n) *orb_n = f->orb_n.data();
    if (names) *names = f->name_ptr.data();
    return BD_OK;
}

// SpProp_t::SpProp_t(char*, ModSpace_t*) (source/BcDor-Sp_Propagator.cpp:387-610); the
// amplitude rows have the model space's largest subshell size as stride.
int bd_files_read_propagator(bd_files *f, const char *path) {
    if (!f || !path) return BD_ERR_ARG;
    if (f->nsubsh < 1) return ffail(f, BD_ERR_STATE, "no model space");
    TextFile t;
    if (!t.load(path)) return ffail(f, BD_ERR_ARG, "propagator '%s': cannot read the file", path);
    t.index();
    size_t k = 4;
    int n1 = 0, nspb_file = 0, wcode = 0;
    {
        const std::string s = t.line(k++);
        const char *p = s.c_str();
        if (!scan_lit(p, "#") || !scan_int(p, n1) || !scan_int(p, nspb_file)) return ffail(f, BD_ERR_ARG, "propagator '%s': line 5", path);
        if (!scan_int(p, wcode)) wcode = 0;
    }
    if (n1 != f->nsubsh)
        return ffail(f, BD_ERR_ARG, "propagator '%s': %d subshells, the model space has %d", path, n1, f->nsubsh);
    const int rw_d1 = wcode % 2, rw_n2 = (wcode / 2) % 2, rw_n1 = (wcode / 4) % 2;
    k += 3;   // blank, "# Total numbers", the totals (counted again below)
    int nspb = 0;
    for (int v : f->no) nspb = std::max(nspb, v);
    std::vector<int> np(f->nsubsh), nh(f->nsubsh);
    std::vector<double> ep, eh, zp, zh, fqp, fqh;
    for (int i = 0; i < f->nsubsh; ++i) {
        k += 3;   // blank, "# Subshell:", "# name"
        for (int side = 0; side < 2; ++side) {
            std::string s = t.line(k++);
            const char *p = s.c_str();
            int n = 0;
            if (!scan_lit(p, "#") || !scan_int(p, n) || n < 0)
                return ffail(f, BD_ERR_ARG, "propagator '%s': fragment count of subshell %d", path, i);
            (side == 0 ? np : nh)[i] = n;
            for (int j = 0; j < n; ++j) {
                s = t.line(k++);
                p = s.c_str();
                double e, z, x;
                int iv;
                if (!scan_dbl(p, e) || !scan_dbl(p, z))
                    return ffail(f, BD_ERR_ARG, "propagator '%s': fragment %d of subshell %d", path, j, i);
                if (rw_n1 && !scan_int(p, iv)) return ffail(f, BD_ERR_ARG, "propagator '%s': n1 column", path);
                if (rw_n2 && !scan_int(p, iv)) return ffail(f, BD_ERR_ARG, "propagator '%s': n2 column", path);
                if (rw_d1 && !scan_dbl(p, x)) return ffail(f, BD_ERR_ARG, "propagator '%s': d1 column", path);
                (side == 0 ? ep : eh).push_back(e);
                (side == 0 ? zp : zh).push_back(z / 100.0);
                std::vector<double> &F = side == 0 ? fqp : fqh;
                const size_t r0 = F.size();
                F.resize(r0 + nspb, 0.0);
                for (int q = 0; q < f->no[i]; ++q) {
                    if (!scan_dbl(p, x)) x = 0.0;   // a missing amplitude reads as zero
                    F[r0 + q] = x;
                }
            }
        }
    }
    f->nspb = nspb;
    f->np.swap(np); f->nh.swap(nh);
    f->ep.swap(ep); f->eh.swap(eh); f->zp.swap(zp); f->zh.swap(zh); f->fqp.swap(fqp); f->fqh.swap(fqh);
    f->have_prop = true;
    return BD_OK;
}

int bd_files_propagator(const bd_files *f, bd_propagator *prop, const double **zp, const double **zh) {
    if (!f || !prop || !f->have_prop) return BD_ERR_STATE;
    static const double zero[8] = {0};
    prop->nspb = f->nspb;
    prop->np = f->np.data(); prop->nh = f->nh.data();
    prop->ep = f->ep.empty() ? zero : f->ep.data();
    prop->eh = f->eh.empty() ? zero : f->eh.data();
    prop->fqp = f->fqp.empty() ? zero : f->fqp.data();
    prop->fqh = f->fqh.empty() ? zero : f->fqh.data();
    if (zp) *zp = f->zp.data();
    if (zh) *zh = f->zh.data();
    return BD_OK;
}

// Make_LancPivots for every subshell (source/BcDor-Miscellanea.cpp:334-390): a
// subshell's pivots are the lines after the first "shell,npvts:  ish  n" header that
// names it; lines without the two iteration counts are skipped; a subshell without a
// header has no pivots.
int bd_files_read_pivots(bd_files *f, const char *path) {
    if (!f || !path) return BD_ERR_ARG;
    if (f->nsubsh < 1) return ffail(f, BD_ERR_STATE, "no model space");
    TextFile t;
    if (!t.load(path)) return ffail(f, BD_ERR_ARG, "pivots '%s': cannot read the file", path);
    t.index();
    std::vector<int> npvt(f->nsubsh, 0), nfw, nbk;
    std::vector<std::vector<int>> sfw(f->nsubsh), sbk(f->nsubsh);
    std::vector<std::vector<double>> svec(f->nsubsh);
    std::vector<char> seen(f->nsubsh, 0);
    for (size_t k = 0; k < t.start.size(); ++k) {
        const std::string s = t.line(k);
        const char *p = s.c_str();
        int ish = 0, n = 0;
        if (!scan_lit(p, "shell,npvts:") || !scan_int(p, ish) || !scan_int(p, n)) continue;
        if (ish < 0 || ish >= f->nsubsh || seen[ish]) continue;
        seen[ish] = 1;
        const int D = f->no[ish];
        for (int i = 0; i < n && k + 1 < t.start.size(); ++i) {
            const std::string r = t.line(++k);
            const char *q = r.c_str();
            int a, b;
            if (!scan_int(q, a) || !scan_int(q, b)) continue;
            std::vector<double> v(D);
            for (int d = 0; d < D; ++d)
                if (!scan_dbl(q, v[d])) return ffail(f, BD_ERR_ARG, "pivots '%s': line %zu has fewer than %d amplitudes", path, k + 1, D);
            sfw[ish].push_back(a); sbk[ish].push_back(b);
            svec[ish].insert(svec[ish].end(), v.begin(), v.end());
            ++npvt[ish];
        }
    }
    std::vector<double> vec;
    for (int i = 0; i < f->nsubsh; ++i) {
        nfw.insert(nfw.end(), sfw[i].begin(), sfw[i].end());
        nbk.insert(nbk.end(), sbk[i].begin(), sbk[i].end());
        vec.insert(vec.end(), svec[i].begin(), svec[i].end());
    }
    f->npvt.swap(npvt); f->nfw.swap(nfw); f->nbk.swap(nbk); f->pvec.swap(vec);
    f->have_piv = true;
    return BD_OK;
}

int bd_files_pivots(const bd_files *f, bd_pivots *piv) {
    if (!f || !piv || !f->have_piv) return BD_ERR_STATE;
    static const int izero[1] = {0};
    static const double dzero[1] = {0.0};
    piv->npvt = f->npvt.data();
    piv->n_itr_fw = f->nfw.empty() ? izero : f->nfw.data();
    piv->n_itr_bk = f->nbk.empty() ? izero : f->nbk.data();
    piv->vec = f->pvec.empty() ? dzero : f->pvec.data();
    return BD_OK;
}

// VppInt_t::read (source/BcDor-Vpp_potential.cpp:205-215): read_bin (:406-438) for a name
// containing ".bin", else read_ascii (:281-375).  The text lines are parsed on `threads`
// host threads; a line naming an orbit outside the model space is skipped and one with
// a Pauli-forbidden pair (a == b or c == d at odd J) is discarded, as read_ascii does.
int bd_files_read_interaction(bd_files *f, const char *path, int threads) {
    if (!f || !path) return BD_ERR_ARG;
    if (f->nsubsh < 1) return ffail(f, BD_ERR_STATE, "no model space");
    f->have_vpp = false;
    f->vabcd.clear(); f->vJ.clear(); f->vV.clear();
    f->n_outside = f->n_pauli = 0;
    if (std::strstr(path, ".bin")) {
        FILE *fp = std::fopen(path, "rb");
        if (!fp) return ffail(f, BD_ERR_ARG, "interaction '%s': cannot read the file", path);
        int dims[6];
        bool ok = std::fread(dims, sizeof(int), 6, fp) == 6 && dims[0] >= 0 && dims[2] >= 0;
        std::vector<double> stren(ok ? dims[2] : 0);
        std::vector<int> iab(ok ? dims[0] : 0), icd(ok ? dims[0] : 0);
        if (ok && dims[2] > 0) ok = std::fread(stren.data(), sizeof(double), dims[2], fp) == (size_t)dims[2];
        if (ok && dims[0] > 0) ok = std::fread(iab.data(), sizeof(int), dims[0], fp) == (size_t)dims[0] &&
                                    std::fread(icd.data(), sizeof(int), dims[0], fp) == (size_t)dims[0];
        int isel = ok ? dims[4] : 0;
        if (isel < 0 || isel >= (ok ? dims[2] : 1)) isel = 0;   // select(): out of range -> 0
        std::vector<double> V(ok ? dims[0] : 0);
        for (int q = 0; ok && q < dims[2]; ++q) {
            std::vector<double> tmp(dims[0]);
            if (dims[0] > 0 && std::fread(tmp.data(), sizeof(double), dims[0], fp) != (size_t)dims[0]) ok = false;
            if (q == isel) V.swap(tmp);
        }
        std::fclose(fp);
        if (!ok || dims[2] < 1) return ffail(f, BD_ERR_ARG, "interaction '%s': truncated or empty binary file", path);
        for (int i = 0; i < dims[0]; ++i) {
            const int J = iab[i] % kJMult, a = (iab[i] / kJMult) / kABMult, b = (iab[i] / kJMult) % kABMult;
            const int J2 = icd[i] % kJMult, c = (icd[i] / kJMult) / kABMult, d = (icd[i] / kJMult) % kABMult;
            if (a >= f->norb || b >= f->norb || c >= f->norb || d >= f->norb || J != J2 || iab[i] < 0 || icd[i] < 0)
                return ffail(f, BD_ERR_ARG, "interaction '%s': element %d has keys outside the model space", path, i);
            f->vabcd.push_back(make_int4(a, b, c, d));
            f->vJ.push_back(J);
        }
        f->vV.swap(V);
        f->n_alloc = dims[1];
        f->have_vpp = true;
        return BD_OK;
    }
    TextFile t;
    if (!t.load(path)) return ffail(f, BD_ERR_ARG, "interaction '%s': cannot read the file", path);
    int nlines = 0;
    {
        const size_t e = t.data.find('\n');
        const std::string first = t.data.substr(0, e == std::string::npos ? t.data.size() : e);
        const char *p = first.c_str();
        if (!scan_int(p, nlines) || nlines < 0) return ffail(f, BD_ERR_ARG, "interaction '%s': no line count on line 1", path);
        t.index(e == std::string::npos ? t.data.size() : e + 1, (size_t)nlines);
    }
    if ((long long)t.start.size() < nlines)
        return ffail(f, BD_ERR_ARG, "interaction '%s': %zu lines after the first, %d declared", path, t.start.size(), nlines);
    // orbit of (n, 2j, parity, charge): ModSpace_t::get_orbit (source/BcDor-Mod_Space.cpp:567-575)
    std::map<std::tuple<int, int, int, int>, int> orbit;
    for (int o = f->norb - 1; o >= 0; --o) {   // the first match wins
        const int s = f->orb_sh[o];
        orbit[std::make_tuple(f->orb_n[o], f->j2[s], f->ip[s], f->ch[s])] = o;
    }
    const int nt = std::max(1, std::min(threads > 0 ? threads : (int)std::thread::hardware_concurrency(), 64));
    struct Part {
        std::vector<int4> abcd;
        std::vector<int> J;
        std::vector<double> V;
        long long outside = 0, pauli = 0, bad = -1;
    };
    std::vector<Part> parts(nt);
    auto work = [&](int w) {
        Part &P = parts[w];
        const long long l0 = (long long)nlines * w / nt, l1 = (long long)nlines * (w + 1) / nt;
        for (long long i = l0; i < l1; ++i) {
            const size_t a0 = t.start[i];
            const char *p = t.data.c_str() + a0;
            int o[4], J = 0;
            bool inside = true, ok = true;
            for (int q = 0; q < 4 && ok; ++q) {
                int n, j2, ip, ch;
                ok = scan_int(p, n) && scan_int(p, j2) && scan_int(p, ip) && scan_int(p, ch);
                if (!ok) break;
                const auto it = orbit.find(std::make_tuple(n, j2, ip % 2, ch));
                if (it == orbit.end()) inside = false;
                else o[q] = it->second;
                if (!inside) break;   // read_line_Vpp returns at the first unknown orbit
            }
            if (ok && !inside) { ++P.outside; continue; }
            double V = 0.0;
            if (!ok || !scan_int(p, J) || !scan_dbl(p, V)) { if (P.bad < 0) P.bad = i; continue; }
            const bool pauli = (o[0] == o[1] && std::abs(f->j2[f->orb_sh[o[0]]] - J) % 2 == 0) ||
                               (o[2] == o[3] && std::abs(f->j2[f->orb_sh[o[2]]] - J) % 2 == 0);
            if (pauli) { ++P.pauli; continue; }
            P.abcd.push_back(make_int4(o[0], o[1], o[2], o[3]));
            P.J.push_back(J);
            P.V.push_back(V);
        }
    };
    std::vector<std::thread> th;
    for (int w = 1; w < nt; ++w) th.emplace_back(work, w);
    work(0);
    for (auto &x : th) x.join();
    size_t tot = 0;
    for (auto &P : parts) {
        if (P.bad >= 0) return ffail(f, BD_ERR_ARG, "interaction '%s': line %lld cannot be read", path, P.bad + 2);
        tot += P.V.size();
    }
    f->vabcd.reserve(tot); f->vJ.reserve(tot); f->vV.reserve(tot);
    for (auto &P : parts) {
        f->vabcd.insert(f->vabcd.end(), P.abcd.begin(), P.abcd.end());
        f->vJ.insert(f->vJ.end(), P.J.begin(), P.J.end());
        f->vV.insert(f->vV.end(), P.V.begin(), P.V.end());
        f->n_outside += P.outside;
        f->n_pauli += P.pauli;
    }
    f->n_alloc = nlines;
    f->have_vpp = true;
    return BD_OK;
}

int bd_files_interaction_lines(const bd_files *f, long long *kept, long long *outside, long long *pauli) {
    if (!f || !f->have_vpp) return BD_ERR_STATE;
    if (kept) *kept = (long long)f->vV.size();
    if (outside) *outside = f->n_outside;
    if (pauli) *pauli = f->n_pauli;
    return BD_OK;
}

// SpProp_t::write with wcode 0 (source/BcDor-Sp_Propagator.cpp:613-680).  zp / zh NULL:
// Z = sum of the squared amplitudes, the value add_qp / add_qh store.
int bd_files_write_propagator(const bd_files *f, const char *path, const bd_propagator *prop, const double *zp,
                              const double *zh) {
    if (!f || !path || !prop) return BD_ERR_ARG;
    if (f->nsubsh < 1) return BD_ERR_STATE;
    FILE *fp = std::fopen(path, "w");
    if (!fp) return BD_ERR_ARG;
    long long nqp = 0, nqh = 0;
    for (int i = 0; i < f->nsubsh; ++i) { nqp += prop->np[i]; nqh += prop->nh[i]; }
    std::fprintf(fp, "#  Quasi- particle and hole fragments of the sp propagator\n");
    std::fprintf(fp, "#----------------------------------------------------------\n");
    std::fprintf(fp, "\n# number of (ilj\\pi) subshells, max n. of radial orbitals:\n");
    std::fprintf(fp, "# %7i %7i %7i\n", f->nsubsh, prop->nspb, 0);
    std::fprintf(fp, "\n# Total numbers of qp and qh stored here:\n");
    std::fprintf(fp, "# %7i %7i\n", (int)nqp, (int)nqh);
    long long kp = 0, kh = 0;
    for (int i = 0; i < f->nsubsh; ++i) {
        std::fprintf(fp, "\n# Subshell:\n");
        std::fprintf(fp, "# %s \n", f->names[i].c_str());
        for (int side = 0; side < 2; ++side) {
            const int n = side == 0 ? prop->np[i] : prop->nh[i];
            std::fprintf(fp, side == 0 ? "# %7i  # -> tot n. of quasiparticles\n" : "# %7i  # -> tot n. of quasiholes\n", n);
            for (int j = 0; j < n; ++j) {
                const long long r = side == 0 ? kp++ : kh++;
                const double *amp = (side == 0 ? prop->fqp : prop->fqh) + (size_t)r * prop->nspb;
                double z = 0.0;
                const double *zz = side == 0 ? zp : zh;
                if (zz) z = zz[r];
                else for (int q = 0; q < f->no[i]; ++q) z += amp[q] * amp[q];
                std::fprintf(fp, " %15.6lf ", (side == 0 ? prop->ep : prop->eh)[r]);
                std::fprintf(fp, " %12.3lf   ", 100. * z);
                for (int q = 0; q < f->no[i]; ++q) std::fprintf(fp, " %18.6le ", amp[q]);
                std::fprintf(fp, "\n");
            }
        }
    }
    return std::fclose(fp) == 0 ? BD_OK : BD_ERR_ARG;
}

// SpProp_t::DysPivots (source/BcDor-Sp_Propagator.cpp:1225-1290): per subshell the
// quasiholes, then the quasiparticles, with 100 Z >= z_cut, by ascending energy (one
// pivot per distinct energy, the first fragment of it in the propagator's order).
int bd_files_write_pivots(const bd_files *f, const char *path, const bd_propagator *prop, const double *zp,
                          const double *zh, int n_fw, int n_bk, double z_cut) {
    if (!f || !path || !prop) return BD_ERR_ARG;
    if (f->nsubsh < 1) return BD_ERR_STATE;
    FILE *fp = std::fopen(path, "w");
    if (!fp) return BD_ERR_ARG;
    std::fprintf(fp, "#   Template pivots file\n");
    std::fprintf(fp, "#\n");
    std::fprintf(fp, "# number of (ilj\\pi) subshells, max n. of radial orbitals:\n");
    std::fprintf(fp, "# %7i %7i\n\n", f->nsubsh, prop->nspb);
    long long p0 = 0, h0 = 0;
    for (int i = 0; i < f->nsubsh; ++i) {
        std::fprintf(fp, "\n\nshell,npvts:   %i   %i  # %s \n", i, f->no[i], f->names[i].c_str());
        for (int side = 1; side >= 0; --side) {   // holes first
            const int n = side == 0 ? prop->np[i] : prop->nh[i];
            const long long b = side == 0 ? p0 : h0;
            const double *E = side == 0 ? prop->ep : prop->eh;
            const double *F = side == 0 ? prop->fqp : prop->fqh;
            const double *Zs = side == 0 ? zp : zh;
            auto Zof = [&](int j) {
                if (Zs) return Zs[b + j];
                double z = 0.0;
                for (int q = 0; q < f->no[i]; ++q) z += F[(size_t)(b + j) * prop->nspb + q] * F[(size_t)(b + j) * prop->nspb + q];
                return z;
            };
            double x2 = -1.0e+10;
            int itest = n < 1 ? -100 : 1;
            while (itest >= 0) {
                itest = -100;
                double x1 = +1.0e+10;
                for (int j = 0; j < n; ++j)
                    if (E[b + j] < x1 && E[b + j] > x2 && 100. * Zof(j) >= z_cut) { x1 = E[b + j]; itest = j; }
                if (itest >= 0) {
                    x2 = x1;
                    std::fprintf(fp, " %3i  %3i  ", n_fw, n_bk);
                    for (int q = 0; q < f->no[i]; ++q) std::fprintf(fp, " %18.6le ", F[(size_t)(b + itest) * prop->nspb + q]);
                    std::fprintf(fp, side == 1 ? "   #    e- = %13.6lf\n" : "   #    e+ = %13.6lf\n", E[b + itest]);
                }
            }
        }
        p0 += prop->np[i];
        h0 += prop->nh[i];
    }
    return std::fclose(fp) == 0 ? BD_OK : BD_ERR_ARG;
}

// VppInt_t::write_bin (source/BcDor-Vpp_potential.cpp:377-404) for one interaction:
// n_me, n_alloc (the allocation the list came from; <= 0 means n_me), one interaction
// selected, its strength slot 0.
int bd_write_interaction_bin(const char *path, const bd_interaction *vpp, long long n_alloc) {
    if (!path || !vpp || vpp->n_me < 0) return BD_ERR_ARG;
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return BD_ERR_ARG;
    const int dims[6] = {vpp->n_me, (int)(n_alloc > 0 ? n_alloc : vpp->n_me), 1, 1, 0, -100};
    const double stren = 0.0;
    bool ok = std::fwrite(dims, sizeof(int), 6, fp) == 6 && std::fwrite(&stren, sizeof(double), 1, fp) == 1;
    if (vpp->n_me > 0)
        ok = ok && std::fwrite(vpp->iabJ, sizeof(int), vpp->n_me, fp) == (size_t)vpp->n_me &&
             std::fwrite(vpp->icdJ, sizeof(int), vpp->n_me, fp) == (size_t)vpp->n_me &&
             std::fwrite(vpp->V, sizeof(double), vpp->n_me, fp) == (size_t)vpp->n_me;
    return (std::fclose(fp) == 0 && ok) ? BD_OK : BD_ERR_ARG;
}

// The reference's file name of a channel's self-energy (Wide_self_energy_t::get_filename,
// source/BcDor-Self_energy_ext_Op_d.cpp:43-52, with Lambda = parity = charge = 0):
// dir/label_Dyn_J2pi=<2j><+|->_dt=<charge>.bin
int bd_files_selfenergy_name(const bd_files *f, const char *dir, const char *label, int ish, char *buf, int len) {
    if (!f || !buf || len < 1 || ish < 0 || ish >= f->nsubsh) return BD_ERR_ARG;
    const int n = std::snprintf(buf, (size_t)len, "%s/%s_%s_J2pi=%i%c_dt=%i.bin", dir ? dir : ".", label ? label : "SelfEn",
                                "Dyn", f->j2[ish], f->ip[ish] % 2 ? '-' : '+', f->ch[ish]);
    return (n >= 0 && n < len) ? BD_OK : BD_ERR_CAPACITY;
}

// Wide_self_energy_t::save_SelfEn_bin (source/BcDor-Self_energy_ext_Op_d.cpp:55-133) for
// the self-energy of channel ish (one partial wave): nden leading doubles per row (2 for
// a plain Sigma(2), n_pvt + 1 for Lanczos rows with their i_piv arrays; NULL ipiv marks
// plain rows).  fwbk > 0 writes only the forward rows, < 0 only the backward ones.
int bd_files_save_selfenergy(const bd_files *f, const char *path, int ish, int nden, int n_fw, const double *fw_rows,
                             const int *ipiv_fw, int n_bk, const double *bk_rows, const int *ipiv_bk, int fwbk) {
    if (!f || !path || ish < 0 || ish >= f->nsubsh || nden < 2 || n_fw < 0 || n_bk < 0) return BD_ERR_ARG;
    const int D = f->no[ish], NDIM = nden + D;
    const bool lz_fw = ipiv_fw && ipiv_fw[0] > 0, lz_bk = ipiv_bk && ipiv_bk[0] > 0;
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return BD_ERR_ARG;
    std::vector<int> h;
    h.push_back(fwbk < 0 ? 0 : n_fw);
    h.push_back(fwbk > 0 ? 0 : n_bk);
    h.push_back(std::max(1, n_fw));   // the allocations the reference's build makes
    h.push_back(std::max(1, n_bk));
    h.push_back(ish); h.push_back(nden); h.push_back(D); h.push_back(NDIM); h.push_back(1);
    h.push_back(f->j2[ish]); h.push_back(f->ip[ish]); h.push_back(f->ch[ish]);
    h.push_back(ish); h.push_back(0); h.push_back(D);                                   // i_pwv, nst_pwv, norb_pwv
    for (int q = 0; q < D; ++q) h.push_back(f->orb_start[ish] + q);                      // isp_msp
    for (int q = 0; q < D; ++q) h.push_back(f->orb_n[f->orb_start[ish] + q]);            // Mor_n
    int n1 = 0;
    if (lz_fw) n1 = std::max(n1, ipiv_fw[0] + 3);
    if (lz_bk) n1 = std::max(n1, ipiv_bk[0] + 3);
    h.push_back(n1); h.push_back(lz_fw ? 1 : 0); h.push_back(lz_bk ? 1 : 0);
    bool ok = std::fwrite(h.data(), sizeof(int), h.size(), fp) == h.size();
    auto block = [&](int n, const double *rows, const int *ipiv, bool lz) {
        if (n > 0) ok = ok && std::fwrite(rows, sizeof(double), (size_t)n * NDIM, fp) == (size_t)n * NDIM;
        if (lz) {
            ok = ok && std::fwrite(&n, sizeof(int), 1, fp) == 1;
            ok = ok && std::fwrite(ipiv, sizeof(int), (size_t)ipiv[0] + 2, fp) == (size_t)ipiv[0] + 2;
        }
    };
    if (fwbk >= 0) block(n_fw, fw_rows, ipiv_fw, lz_fw);
    if (fwbk <= 0) block(n_bk, bk_rows, ipiv_bk, lz_bk);
    return (std::fclose(fp) == 0 && ok) ? BD_OK : BD_ERR_ARG;
}

// Wide_self_energy_t::load_SelfEn_bin for one file (source/BcDor-Self_energy_ext_Op_d.cpp:
// 136-210, 213-255): the header is checked against the model space's channel ish; the
// rows and i_piv arrays land in the caller's buffers (NULL buffers: sizes only).
int bd_files_load_selfenergy(const bd_files *f, const char *path, int ish, int *nden, int *n_fw, double *fw_rows,
                             int cap_fw, int *ipiv_fw, int *n_bk, double *bk_rows, int cap_bk, int *ipiv_bk) {
    if (!f || !path || ish < 0 || ish >= f->nsubsh) return BD_ERR_ARG;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return ffail(const_cast<bd_files *>(f), BD_ERR_ARG, "self-energy '%s': cannot read the file", path);
    auto bad = [&](const char *what) {
        std::fclose(fp);
        return ffail(const_cast<bd_files *>(f), BD_ERR_ARG, "self-energy '%s': %s", path, what);
    };
    int h[15];
    if (std::fread(h, sizeof(int), 12, fp) != 12) return bad("short header");
    const int D = f->no[ish];
    if (h[4] != ish || h[9] != f->j2[ish] || h[10] != f->ip[ish] || h[11] != f->ch[ish]) return bad("another channel");
    if (h[6] != D || h[8] != 1) return bad("orbit count or partial waves differ from the model space");
    if (h[5] < 2 || h[7] != h[5] + D || h[0] < 0 || h[1] < 0) return bad("row layout");
    std::vector<int> tab(3 + 2 * D);
    if (std::fread(tab.data(), sizeof(int), tab.size(), fp) != tab.size()) return bad("short partial-wave table");
    if (tab[0] != ish || tab[1] != 0 || tab[2] != D) return bad("partial-wave table");
    for (int q = 0; q < D; ++q)
        if (tab[3 + q] != f->orb_start[ish] + q || tab[3 + D + q] != f->orb_n[f->orb_start[ish] + q]) return bad("orbit list");
    if (std::fread(h + 12, sizeof(int), 3, fp) != 3) return bad("short block header");
    if ((h[13] != 0 && h[13] != 1) || (h[14] != 0 && h[14] != 1)) return bad("more than one Lanczos block");
    const int NDIM = h[7];
    if (nden) *nden = h[5];
    if (n_fw) *n_fw = h[0];
    if (n_bk) *n_bk = h[1];
    if ((fw_rows && cap_fw < h[0]) || (bk_rows && cap_bk < h[1])) { std::fclose(fp); return BD_ERR_CAPACITY; }
    for (int side = 0; side < 2; ++side) {
        const int n = h[side];
        double *rows = side == 0 ? fw_rows : bk_rows;
        int *ipiv = side == 0 ? ipiv_fw : ipiv_bk;
        std::vector<double> tmp;
        double *dst = rows;
        if (!dst) { tmp.resize((size_t)n * NDIM); dst = tmp.data(); }
        if (n > 0 && std::fread(dst, sizeof(double), (size_t)n * NDIM, fp) != (size_t)n * NDIM) return bad("short rows");
        if (ipiv) for (int q = 0; q < NDIM; ++q) ipiv[q] = 0;
        if (h[13 + side] > 0) {
            int nr = 0, nu = 0;
            if (std::fread(&nr, sizeof(int), 1, fp) != 1 || std::fread(&nu, sizeof(int), 1, fp) != 1) return bad("short i_piv");
            if (nu < 0 || nu + 2 > NDIM) return bad("i_piv longer than a row");
            std::vector<int> ip(nu + 2);
            ip[0] = nu;
            if (std::fread(ip.data() + 1, sizeof(int), nu + 1, fp) != (size_t)nu + 1) return bad("short i_piv");
            if (ipiv) for (int q = 0; q < nu + 2; ++q) ipiv[q] = ip[q];
        }
    }
    std::fclose(fp);
    return BD_OK;
}

}  // extern "C"

// ------------------------------------------------------------------- device canonical list
namespace bd {

bool files_interaction(const bd_files *f, const int4 **abcd, const int **J, const double **V, long long *n) {
    if (!f || !f->have_vpp) return false;
    *abcd = f->vabcd.data();
    *J = f->vJ.data();
    *V = f->vV.data();
    *n = (long long)f->vV.size();
    return true;
}

// read_ascii's canonical form of one line (source/BcDor-Vpp_potential.cpp:330-356): the
// pairs ordered a <= b and c <= d, each swap a phase (-1)^(j_a + j_b - J + 1) (2j / 2
// units), then the two pair keys ordered; and prepare_for_reading's key (charge sum,
// parity, J) of the pair ab, which must equal cd's (:451-468).  The sort key puts the
// list in prepare_for_reading's order: (ch, pi, J) segment, then iabJ, then icdJ; in a
// segment J is fixed, so the orbit pairs order the keys.  val = the line's index.
__global__ void k_vpp_canon(const int4 *abcd, const int *Jv, long long n, const int *orb_sh, const int *j2,
                            const int *ip, const int *ch, unsigned long long *key, unsigned *val, signed char *sign,
                            int *bad) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 o = abcd[i];
    const int J = Jv[i];
    int a = o.x, b = o.y, c = o.z, d = o.w, iph = 0;
    if (a > b) { iph += (j2[orb_sh[a]] + j2[orb_sh[b]]) / 2 - J + 1; const int t = a; a = b; b = t; }
    if (c > d) { iph += (j2[orb_sh[c]] + j2[orb_sh[d]]) / 2 - J + 1; const int t = c; c = d; d = t; }
    if (a * kABMult + b > c * kABMult + d) { int t = a; a = c; c = t; t = b; b = d; d = t; }
    const int sa = orb_sh[a], sb = orb_sh[b], sc = orb_sh[c], sd = orb_sh[d];
    const int cab = ch[sa] + ch[sb], pab = (ip[sa] + ip[sb]) % 2;
    if (cab != ch[sc] + ch[sd] || pab != (ip[sc] + ip[sd]) % 2 || J < 0 || J >= kJMult || cab - kChOff < 0 ||
        cab - kChOff >= kChMult)
        atomicMax(bad, (int)min(i + 1, (long long)INT_MAX));
    const unsigned long long seg = (unsigned long long)ind_chipJ(cab, pab, J) & 0x7ffull;
    key[i] = (seg << 40) | ((unsigned long long)a << 30) | ((unsigned long long)b << 20) | ((unsigned long long)c << 10) |
             (unsigned long long)d;
    val[i] = (unsigned)i;
    sign[i] = (signed char)((abs(iph) % 2) ? -1 : 1);
}

// Repeated keys after the sort: check_for_double_entries keeps the first of each run
// (source/BcDor-Vpp_potential.cpp:663-702).  keep[i] = 1 for the first of its key.
__global__ void k_vpp_first(const unsigned long long *key, long long n, unsigned *keep) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    keep[i] = (i == 0 || key[i] != key[i - 1]) ? 1u : 0u;
}

// The kept pairs at their places in the list: iabJ, icdJ and V with the line's phase.
__global__ void k_vpp_place(const unsigned long long *key, const unsigned *val, const unsigned *pos, const unsigned *keep,
                            long long n, const double *Vin, const signed char *sign, int *iabJ, int *icdJ, double *V) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n || !keep[i]) return;
    const unsigned long long k = key[i];
    const int J = (int)((k >> 40) & 0x7ffull) % kJMult;
    const int a = (int)((k >> 30) & 1023ull), b = (int)((k >> 20) & 1023ull), c = (int)((k >> 10) & 1023ull),
              d = (int)(k & 1023ull);
    const unsigned p = pos[i];
    iabJ[p] = ind_i1i2J(a, b, J);
    icdJ[p] = ind_i1i2J(c, d, J);
    const unsigned src = val[i];
    V[p] = sign[src] < 0 ? -Vin[src] : Vin[src];
}

}  // namespace bd
