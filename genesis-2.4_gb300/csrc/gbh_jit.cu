// gbh_jit.cu -- per-program kernel specialisation at setup.
//
// The interpreting kernels (k_steps, k_steps_mixed) read each compartment's
// micro-ops from memory, so every load of a compartment waits for the
// opcode before it and little memory-level parallelism is exposed. For a
// tile type (all neurons sharing one program) this file emits the same
// computation as straight-line CUDA -- every slot unrolled, every field row,
// table column, power and stablist index a literal, the elimination unrolled
// in registers when all neurons of the type share one tree -- and compiles
// it with NVRTC for the running GPU. The arithmetic of each micro-op is
// emitted exactly as the interpreter performs it, so the FP64 form stays
// bit-identical (it is compiled without multiply-add contraction).
//
// NVRTC is loaded with dlopen and the driver calls are resolved through
// cudaGetDriverEntryPointByVersion, so the library links neither.
#include "gbh_jit.h"

#include <cuda.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <cstdio>
#include <array>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <sstream>

#include "gbh_internal.h"
#include "gbh_jit_sources.h"   // generated at build time: header texts

namespace gbh {

namespace {

// ---- NVRTC and driver entry points ----------------------------------------
struct Api {
    bool ok = false;
    std::string why;
    nvrtcResult (*create)(nvrtcProgram *, const char *, const char *, int, const char *const *,
                          const char *const *) = nullptr;
    nvrtcResult (*compile)(nvrtcProgram, int, const char *const *) = nullptr;
    nvrtcResult (*logsize)(nvrtcProgram, size_t *) = nullptr;
    nvrtcResult (*getlog)(nvrtcProgram, char *) = nullptr;
    nvrtcResult (*cubinsize)(nvrtcProgram, size_t *) = nullptr;
    nvrtcResult (*getcubin)(nvrtcProgram, char *) = nullptr;
    nvrtcResult (*destroy)(nvrtcProgram *) = nullptr;
    CUresult (*load)(CUmodule *, const void *) = nullptr;
    CUresult (*getfn)(CUfunction *, CUmodule, const char *) = nullptr;
    CUresult (*launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                       CUstream, void **, void **) = nullptr;
    CUresult (*setattr)(CUfunction, CUfunction_attribute, int) = nullptr;
    CUresult (*unload)(CUmodule) = nullptr;
};

Api g_api;
std::once_flag g_api_once;

template <typename F>
bool sym(void *h, const char *name, F &fn)
{
    fn = reinterpret_cast<F>(dlsym(h, name));
    return fn != nullptr;
}

template <typename F>
bool drv(const char *name, F &fn)
{
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 13000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
        return false;
    fn = reinterpret_cast<F>(p);
    return true;
}

void init_api()
{
    const char *cands[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                           "/usr/local/cuda/lib64/libnvrtc.so"};
    void *h = nullptr;
    for (const char *c : cands)
        if ((h = dlopen(c, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) {
        g_api.why = "libnvrtc not found";
        return;
    }
    bool ok = sym(h, "nvrtcCreateProgram", g_api.create) && sym(h, "nvrtcCompileProgram", g_api.compile) &&
              sym(h, "nvrtcGetProgramLogSize", g_api.logsize) && sym(h, "nvrtcGetProgramLog", g_api.getlog) &&
              sym(h, "nvrtcGetCUBINSize", g_api.cubinsize) && sym(h, "nvrtcGetCUBIN", g_api.getcubin) &&
              sym(h, "nvrtcDestroyProgram", g_api.destroy);
    ok = ok && drv("cuModuleLoadData", g_api.load) && drv("cuModuleGetFunction", g_api.getfn) &&
         drv("cuLaunchKernel", g_api.launch) && drv("cuFuncSetAttribute", g_api.setattr) &&
         drv("cuModuleUnload", g_api.unload);
    if (!ok) {
        g_api.why = "NVRTC or driver entry points missing";
        return;
    }
    g_api.ok = true;
}

// ---- source emission -------------------------------------------------------
std::string lit(double x)
{
    char b[64];
    snprintf(b, sizeof(b), "%a", x);
    return b;
}
std::string litf(float x)
{
    char b[64];
    snprintf(b, sizeof(b), "%af", (double)x);
    return b;
}

struct Emit {
    std::ostringstream o;
    bool mixed, giv;
    // inside a loop over a run of slots: the slot index variable and, per
    // field row of the run's first slot, its row as an expression of the loop
    std::string sidx;
    std::map<int, std::string> fx;
    std::string frow(int f) const
    {
        auto it = fx.find(f);
        return it == fx.end() ? std::to_string(f * LANES) : "(" + it->second + ") * 32";
    }
    std::string P(int f) const { return "Pw[" + frow(f) + "]"; }
    std::string I(int r) const { return "Iw[" + std::to_string(r * LANES) + "]"; }
    std::string C(int p) const { return "Cw[" + std::to_string(p * LANES) + "]"; }
    std::string F(int p) const { return "Fw[" + std::to_string(p * LANES) + "]"; }
    std::string G(int g) const { return "Gw[" + std::to_string(g * LANES) + "]"; }
    std::string pP(int f) const { return "&Pw[" + frow(f) + "]"; }
    // rows no op of the kernel writes (chip constants: Em/Rm, inject, tbyc,
    // diagterm, Ek, gmax): non-coherent loads
    std::string Pr(int f) const { return "__ldg(&Pw[" + frow(f) + "])"; }
    std::string ldr(int f) const { return (stream ? "ld_df_stream(&Pw[" : "ld_df_ro(&Pw[") + frow(f) + "])"; }
    bool stream = false;   // unrolled form: each row is read once per step
    std::string S(int s) const { return sidx.empty() ? std::to_string(s) : sidx; }
    std::string Vrow(int s) const { return sidx.empty() ? std::to_string(s * LANES) : sidx + " * 32"; }
};

int nops_of(int code)
{
    switch (code) {
    case M_BEGIN: return 4;
    case M_NEWVOLT: case M_NEWCONC1: case M_FLUX: case M_DO_TABGHK: return 0;
    case M_CONCVAL: case M_DOMAIN: case M_NEWCONC2: case M_SCALE_FLUX: case M_SAME_GHK:
    case M_CHAN_G: case M_ADDCURR: return 1;
    case M_NERNST: case M_CHAN: case M_STORE: return 2;
    case M_SPIKE: case M_GHK: case M_END: case M_ITLEAK: return 3;
    case M_ELMMPUMP: case M_GATE: case M_MGBLOCK: return 4;
    case M_SYN: return 6;
    default: return -1;
    }
}

// One compartment's channel program. Returns false on an unknown op.
bool emit_slot(Emit &E, int s, const int *&pc, const TableGeom &tg)
{
    std::ostringstream &o = E.o;
    const bool mx = E.mixed, giv = E.giv;
    const int ncols = tg.ncols;
    o << "    { // slot " << E.S(s) << "\n";
    o << "      const double Vm = Vw[" << E.Vrow(s) << "];\n";
    if (mx) o << "      const df vmd = d2df(Vm);\n      df sumg = df_make(0.f, 0.f), ichan = sumg;\n";
    else o << "      double sumg = 0.0, ichan = 0.0;\n";
    o << "      double Im = 0.0; (void)Im;\n";
    // state carried inside the compartment
    for (;;) {
        const int code = pc[0];
        const int n = nops_of(code);
        if (n < 0) return false;
        const int *a = pc + 1;
        switch (code) {
        case M_BEGIN:
            if (mx) {
                // the inject row is read coherently: per-step inputs are written into it
                // by the kernel itself (fused host I/O)
                o << "      { const df emrm = " << E.ldr(a[0]) << "; ichan = df_add(emrm, " << (E.stream ? "ld_df_cg(" : "ld_df(")
                  << E.pP(a[1]) << "));";
                if (giv) o << " Im = df2d(emrm) - Vm / " << E.P(a[2]) << "; " << E.G(a[3]) << " = Im;";
                o << " }\n";
            } else {
                o << "      { const double emrm = " << E.Pr(a[0]) << "; ichan = emrm + " << E.P(a[1]) << ";";
                if (giv) o << " Im = emrm - Vm / " << E.P(a[2]) << "; " << E.G(a[3]) << " = Im;";
                o << " }\n";
            }
            break;
        case M_NEWVOLT:
            if (mx)
                o << "      locate_df(vc, vmd, xnmin, xinv, " << tg.xdivs << ", " << ncols << ");\n";
            else
                o << "      locate(vc, Vm, " << lit(tg.xmin) << ", " << lit(tg.invdx) << ", " << tg.xdivs
                  << ", xvals, " << ncols << ", interp);\n";
            break;
        case M_CONCVAL:
            o << "      sel = " << a[0] << "; " << E.F(a[0]) << " = 0.0;\n";
            break;
        case M_DOMAIN:
            if (mx)
                o << "      locate_df(cc, d2df(" << E.P(a[0]) << " * Ik), ynmin, yinv, " << tg.ydivs << ", " << ncols
                  << ");\n";
            else
                o << "      locate(cc, " << E.P(a[0]) << " * Ik, " << lit(tg.ymin) << ", " << lit(tg.invdy) << ", "
                  << tg.ydivs << ", yvals, " << ncols << ", interp); ctab_base = cc.base;\n";
            break;
        case M_NEWCONC2:
            if (mx)
                o << "      c1 = cc; locate_df(cc, d2df(" << E.C(a[0]) << "), ynmin, yinv, " << tg.ydivs << ", "
                  << ncols << ");\n";
            else
                o << "      tab_base = ctab_base; save_frac = cc.frac; locate(cc, " << E.C(a[0]) << ", "
                  << lit(tg.ymin) << ", " << lit(tg.invdy) << ", " << tg.ydivs << ", yvals, " << ncols
                  << ", interp); ctab_base = cc.base;\n";
            break;
        case M_NEWCONC1:
            if (mx)
                o << "      locate_df(cc, d2df(Cw[sel * 32]), ynmin, yinv, " << tg.ydivs << ", " << ncols << ");\n";
            else
                o << "      locate(cc, Cw[sel * 32], " << lit(tg.ymin) << ", " << lit(tg.invdy) << ", " << tg.ydivs
                  << ", yvals, " << ncols << ", interp); ctab_base = cc.base;\n";
            break;
        case M_SPIKE:
            o << "      if (!v.spike_pre) " << E.I(a[1]) << " = spike_op(v, Vm, " << E.P(a[0]) << ", " << E.I(a[1])
              << ", " << E.I(a[2]) << ", active, neuron, step);\n";
            break;
        case M_ELMMPUMP:
            o << "      { const double cx = Cw[sel * 32]; const double X = 1.0 / (cx + " << E.P(a[0])
              << "); const double vmax = " << E.P(a[1]) << "; Ik = vmax * cx * X;";
            if (mx) o << " ichan = df_add(ichan, d2df(Ik));";
            else o << " ichan += Ik;";
            if (giv) o << " " << E.G(a[3]) << " = c5 ? Ik / vmax : Ik;";
            o << " Im += Ik; }\n";
            break;
        case M_FLUX:
            o << "      Fw[sel * 32] += Ik;\n";
            break;
        case M_SCALE_FLUX:
            o << "      Fw[sel * 32] += " << E.P(a[0]) << " * Ik;\n";
            break;
        case M_STORE:
            break;
        case M_END:
            if (mx) {
                o << "      { const df tbyc = " << E.ldr(a[0]) << "; const df dv = df_mul(ichan, tbyc);\n"
                  << "        R[" << E.S(s) << "] = df2d(df_add(vmd, dv));\n"
                  << "        D[" << E.S(s) << "] = df2d(df_add(df_mul(sumg, tbyc), " << E.ldr(a[1]) << ")); }\n";
            } else {
                o << "      { const double tbyc = " << E.Pr(a[0]) << "; R[" << E.S(s) << "] = Vm + ichan * tbyc; D[" << E.S(s)
                  << "] = sumg * tbyc + " << E.Pr(a[1]) << "; }\n";
            }
            if (giv) o << "      " << E.G(a[2]) << " = Im;\n";
            pc += 1 + n;
            o << "    }\n";
            return true;
        default: {
            // current-producing op then its conductance sub-program
            if (code == M_GHK) {
                o << "      { const double cin = Cw[sel * 32], cout = Cw[(sel + 1) * 32]; double g = " << E.P(a[0])
                  << "; const double X = Vm * g; const double Y = exp(-X); double e = " << E.P(a[1])
                  << "; double ik = e * (cin - (Y * cout)); double gk;\n"
                  << "        if (fabs(X) < 1.0e-6) { gk = 1.0 - 0.5 * X; g = 0.5 * g * e * (cin + cout); ik = -ik / gk; }\n"
                  << "        else { gk = 1.0 - Y; g = g * (ik / gk - e * g * (cin - cout) * Vm * Y / (gk * gk)); ik = -X * ik / gk; }\n"
                  << "        GHK = g;";
                if (mx)
                    o << " Ek = d2df((ik + g * Vm) / g); gmax = d2df(" << E.P(a[2]) << "); Gk = d2df(" << E.P(a[2])
                      << " * GHK); }\n";
                else
                    o << " Ek = (ik + g * Vm) / g; gmax = " << E.P(a[2]) << "; Gk = gmax * GHK; }\n";
            } else if (code == M_SAME_GHK) {
                if (mx) o << "      gmax = d2df(" << E.P(a[0]) << "); Gk = d2df(" << E.P(a[0]) << " * GHK);\n";
                else o << "      gmax = " << E.P(a[0]) << "; Gk = gmax * GHK;\n";
            } else if (code == M_DO_TABGHK) {
                o << "      doGHK = 1;\n";
            } else if (code == M_NERNST) {
                if (mx)
                    o << "      Ek = d2df(log(Cw[(sel + 1) * 32] / Cw[sel * 32]) * " << E.P(a[0]) << "); gmax = Gk = d2df("
                      << E.P(a[1]) << ");\n";
                else
                    o << "      Ek = log(Cw[(sel + 1) * 32] / Cw[sel * 32]) * " << E.P(a[0]) << "; gmax = Gk = "
                      << E.P(a[1]) << ";\n";
            } else if (code == M_CHAN) {
                if (mx) o << "      Ek = " << E.ldr(a[0]) << "; gmax = Gk = " << E.ldr(a[1]) << ";\n";
                else o << "      Ek = " << E.Pr(a[0]) << "; gmax = Gk = " << E.Pr(a[1]) << ";\n";
            } else if (code == M_CHAN_G) {
                if (mx) o << "      gmax = Gk = " << E.ldr(a[0]) << ";\n";
                else o << "      gmax = Gk = " << E.Pr(a[0]) << ";\n";
            } else {
                return false;
            }
            pc += 1 + n;
            for (;;) {
                const int k = pc[0];
                const int m = nops_of(k);
                if (m < 0) return false;
                const int *b = pc + 1;
                if (k == M_GATE) {
                    const int kind = b[0], col = b[1], p = b[2], fs = b[3];
                    o << "      {\n";
                    if (mx) {
                        if (kind == GK_1V || kind == GK_1C) {
                            const char *cu = kind == GK_1V ? "vc" : "cc";
                            o << "        const int bb = " << cu << ".base + " << col << ";\n"
                              << "        const df X = interp_df(tab, bb, " << cu << ".frac), Y = interp_df(tab, bb + 1, "
                              << cu << ".frac);\n";
                        } else {
                            const char *ru = kind == GK_2V ? "vc" : "c1";
                            o << "        const int bb = " << ru << ".base + cc.row + cc.row + " << col << ";\n"
                              << "        const df cf = cc.frac, rf = " << ru << ".frac;\n"
                              << "        const df one_c = df_add_f(df_neg(cf), 1.0f), one_r = df_add_f(df_neg(rf), 1.0f);\n"
                              << "        df q[2];\n"
                              << "        for (int h = 0; h < 2; ++h) { const df t00 = val_df(tab, bb + h), t01 = val_df(tab, bb + 2 + h);\n"
                              << "          const df t10 = interp_df(tab, bb + h, df_make(1.f, 0.f)), t11 = interp_df(tab, bb + 2 + h, df_make(1.f, 0.f));\n"
                              << "          q[h] = df_add(df_mul(one_r, df_add(df_mul(one_c, t00), df_mul(cf, t01))), df_mul(rf, df_add(df_mul(one_c, t10), df_mul(cf, t11)))); }\n"
                              << "        const df X = q[0], Y = q[1];\n";
                        }
                        if (p == 0) {
                            o << "        Ek = Y;\n";
                            pc += 1 + m;
                            if (pc[0] != M_ADDCURR) {   // DO_TABGHK: slope conductance, no current
                                o << "        GHK = df2d(X); doGHK = 0;\n      }\n";
                                break;
                            }
                            o << "        Gk = df_mul(Gk, X);\n      }\n";
                            continue;
                        }
                        o << "        double *st = " << E.pP(fs) << ";\n";
                        if (p > 0)
                            o << "        const df x = df_div(df_add(df_mul(ld_df(st), df_add_f(df_neg(X), 2.0f)), Y), X);\n";
                        else
                            o << "        const df x = df_div(Y, X);\n";
                        o << "        st_df(st, x); Gk = dpow(Gk, x, " << (p > 0 ? p : -p) << ");\n      }\n";
                    } else {
                        if (kind == GK_1V || kind == GK_1C) {
                            o << "        const int bb = " << (kind == GK_1V ? "vc.base" : "ctab_base") << " + " << col
                              << ";\n        double X, Y;\n"
                              << "        if (interp) { const double fr = " << (kind == GK_1V ? "vc" : "cc")
                              << ".frac; X = tab[bb]; X = X + fr * (tab[bb + " << ncols << "] - X); Y = tab[bb + 1]; Y = Y + fr * (tab[bb + 1 + "
                              << ncols << "] - Y); }\n        else { X = tab[bb]; Y = tab[bb + 1]; }\n";
                        } else {
                            o << "        const double rf = " << (kind == GK_2V ? "vc.frac" : "save_frac")
                              << ", cf = cc.frac;\n        const int bb = " << (kind == GK_2V ? "vc.base" : "tab_base")
                              << " + cc.row + cc.row + " << col << ";\n        double X, Y;\n"
                              << "        if (interp) { const int nn = bb + " << ncols
                              << ";\n          X = (1.0 - rf) * ((1.0 - cf) * tab[bb] + cf * tab[bb + 2]) + rf * ((1.0 - cf) * tab[nn] + cf * tab[nn + 2]);\n"
                              << "          Y = (1.0 - rf) * ((1.0 - cf) * tab[bb + 1] + cf * tab[bb + 3]) + rf * ((1.0 - cf) * tab[nn + 1] + cf * tab[nn + 3]); }\n"
                              << "        else { X = tab[bb]; Y = tab[bb + 1]; }\n";
                        }
                        o << "        tab_base = bb + 1;\n";
                        if (p == 0) {
                            o << "        Ek = Y;\n";
                            pc += 1 + m;
                            if (pc[0] != M_ADDCURR) {
                                o << "        GHK = X; doGHK = 0;\n      }\n";
                                break;
                            }
                            o << "        Gk *= X;\n      }\n";
                            continue;
                        }
                        o << "        double *st = " << E.pP(fs) << ";\n";
                        if (p > 0) o << "        const double x = (*st * (2.0 - X) + Y) / X;\n";
                        else o << "        const double x = Y / X;\n";
                        o << "        *st = x; Gk = gpow<double>(Gk, x, " << (p > 0 ? p : -p) << ");\n      }\n";
                    }
                    pc += 1 + m;
                    continue;
                } else if (k == M_SYN) {
                    const int ff = b[0], stab = b[1], srow = b[2], fx = b[3], fy = b[4], fw = b[5];
                    o << "      { const double *sl = v.stablist + " << stab << "; double *px = " << E.pP(fx)
                      << "; double *py = " << E.pP(fy) << ";\n";
                    if (ff >= 0)
                        o << "        { const uint64_t key = ((uint64_t)neuron << 24) ^ ((uint64_t)step << 1) ^ (uint64_t)"
                          << fx << "; if (syn3_uniform(key) <= " << E.P(ff) << ") *px += sl[3]; }\n";
                    o << "        double X = *px * sl[0];\n"
                      << "        unsigned *cell = v.ring + ((tl.syn + (int64_t)" << srow
                      << " * v.ring_len + (int64_t)(step % v.ring_len)) * 32 + lane);\n"
                      << "        { double act; if (syn_due(v, cell, " << E.P(fw) << ", step, act)) X += v.dt * act * sl[3]; }\n"
                      << "        *px = X; const double Y = X * sl[1] + *py * sl[2]; *py = Y;";
                    if (mx) o << " Gk = df_mul(Gk, d2df(Y)); }\n";
                    else o << " Gk *= Y; }\n";
                    pc += 1 + m;
                    continue;
                } else if (k == M_MGBLOCK) {
                    o << "      {";
                    if (mx) {
                        o << " const double gk = df2d(Gk), ek = df2d(Ek);";
                        if (giv)
                            o << " { const double gm = c5 ? df2d(gmax) : 1.0; " << E.G(b[3]) << " = gk / gm; "
                              << E.G(b[3] + 1) << " = gk * (ek - Vm) / gm; " << E.G(b[3] + 2) << " = ek; }";
                        o << " const double X = " << E.P(b[0]) << " * exp(Vm * " << E.P(b[1]) << "); Gk = d2df(gk * (X / (X + "
                          << E.P(b[2]) << "))); }\n";
                    } else {
                        if (giv)
                            o << " if (c5) { " << E.G(b[3]) << " = Gk / gmax; " << E.G(b[3] + 1) << " = Gk * (Ek - Vm) / gmax; } else { "
                              << E.G(b[3]) << " = Gk; " << E.G(b[3] + 1) << " = Gk * (Ek - Vm); } " << E.G(b[3] + 2)
                              << " = Ek;";
                        o << " const double X = " << E.P(b[0]) << " * exp(Vm * " << E.P(b[1]) << "); Gk *= X / (X + "
                          << E.P(b[2]) << "); }\n";
                    }
                    pc += 1 + m;
                    continue;
                } else if (k == M_ADDCURR) {
                    const int g = b[0];
                    if (mx) {
                        o << "      { sumg = df_add(sumg, Gk); ichan = df_add(ichan, df_mul(Ek, Gk)); const double gk = df2d(Gk), ek = df2d(Ek); Ik = gk * (ek - Vm);";
                        if (giv)
                            o << " { const double gm = c5 ? df2d(gmax) : 1.0; " << E.G(g) << " = gk / gm; " << E.G(g + 1)
                              << " = Ik / gm; " << E.G(g + 2) << " = ek; }";
                        o << " Im += Ik; }\n";
                    } else {
                        o << "      { sumg += Gk; ichan += Ek * Gk; Ik = Gk * (Ek - Vm);";
                        if (giv)
                            o << " if (c5) { " << E.G(g) << " = Gk / gmax; " << E.G(g + 1) << " = Ik / gmax; } else { "
                              << E.G(g) << " = Gk; " << E.G(g + 1) << " = Ik; } " << E.G(g + 2) << " = Ek;";
                        o << " Im += Ik; }\n";
                    }
                    pc += 1 + m;
                    break;
                } else {
                    return false;
                }
            }
            break;
        }
        }
        if (code != M_GHK && code != M_SAME_GHK && code != M_DO_TABGHK && code != M_NERNST && code != M_CHAN &&
            code != M_CHAN_G)
            pc += 1 + n;
    }
}

// Operand roles of the micro-ops a loop over slots may hold: positions of
// field rows (may vary with the slot), of literals (must be equal), and of
// givals rows (unused without givals). False for any other op.
bool loop_roles(int code, std::vector<int> &fpos, std::vector<int> &fixed)
{
    fpos.clear();
    fixed.clear();
    switch (code) {
    case M_BEGIN: fpos = {0, 1, 2}; return true;
    case M_NEWVOLT: return true;
    case M_CHAN: fpos = {0, 1}; return true;
    case M_CHAN_G: fpos = {0}; return true;
    case M_GATE: fixed = {0, 1, 2}; fpos = {3}; return true;
    case M_ADDCURR: return true;
    case M_END: fpos = {0, 1}; return true;
    default: return false;
    }
}

// Number of consecutive slots from s0 whose programs equal slot s0's op for
// op, literals equal and every field row affine in the slot index; fills
// the first slot's field rows with their strides.
int loop_run(const std::vector<int> &prog, const std::vector<int> &sstart, int s0, int S,
             std::map<int, int> &stride_of)
{
    stride_of.clear();
    const int len = sstart[s0 + 1] - sstart[s0];
    if (s0 + 1 >= S || sstart[s0 + 2] - sstart[s0 + 1] != len) return 1;
    const int *a = prog.data() + sstart[s0];
    const int *b = prog.data() + sstart[s0 + 1];
    std::vector<int> fpos, fixed;
    std::vector<std::pair<int, int>> fr;   // (offset in the slot program, stride)
    for (int o = 0; o < len;) {
        const int code = a[o];
        if (b[o] != code || !loop_roles(code, fpos, fixed)) return 1;
        if (code == M_GATE && a[o + 1] != GK_1V) return 1;
        for (int k : fixed)
            if (a[o + 1 + k] != b[o + 1 + k]) return 1;
        for (int k : fpos) fr.push_back({o + 1 + k, b[o + 1 + k] - a[o + 1 + k]});
        o += 1 + nops_of(code);
    }
    for (auto &x : fr) {
        auto it = stride_of.find(a[x.first]);
        if (it != stride_of.end() && it->second != x.second) return 1;
        stride_of[a[x.first]] = x.second;
    }
    int run = 2;
    for (int j = s0 + 2; j < S; ++j) {
        if (sstart[j + 1] - sstart[j] != len) break;
        const int *c = prog.data() + sstart[j];
        bool same = true;
        for (int o = 0; o < len && same;) {
            const int code = a[o];
            if (c[o] != code) { same = false; break; }
            loop_roles(code, fpos, fixed);
            for (int k : fixed) same = same && c[o + 1 + k] == a[o + 1 + k];
            o += 1 + nops_of(code);
        }
        for (auto &x : fr) same = same && c[x.first] == a[x.first] + (j - s0) * x.second;
        if (!same) break;
        ++run;
    }
    return run;
}

}  // namespace

std::string jit_source(const TileType &tt, const std::vector<int> &prog, const TableGeom &tg, bool mixed, bool giv,
                       const std::vector<int> *uniform_parent, int min_blocks, bool compact, bool smem_rows,
                       int warps)
{
    if (tt.has_cd || tt.nscratch || tt.sym || tt.nitot)   // diffusion, symmetric, storemode: interpreted
        return std::string();
    if (compact) uniform_parent = nullptr;   // rows in shared-memory columns, looped elimination
    const bool cols = !uniform_parent || smem_rows;   // D/R rows in shared-memory columns
    Emit E;
    E.mixed = mixed;
    E.giv = giv;
    std::ostringstream &o = E.o;
    const int S = tt.nslots;
    o << "#include \"gbh_devfn.cuh\"\nusing namespace gbh;\n";
    o << "extern \"C\" __global__ void __launch_bounds__(" << warps * LANES << ", " << min_blocks
      << ") gbh_jit(DevView v, int tile0, int tile1, int smax, int nsteps, long long step0)\n{\n";
    o << "  extern __shared__ double sm[];\n"
      << "  const int lane = threadIdx.x & 31; const int wib = threadIdx.x >> 5;\n"
      << "  const int t = tile0 + blockIdx.x * (blockDim.x >> 5) + wib; if (t >= tile1) return;\n"
      << "  const long long sbase = v.step_dev ? *v.step_dev : 0;\n"
      << "  const Tile tl = v.tiles[t];\n"
      << "  const bool active = lane < tl.nlanes; (void)active;\n"
      << "  const bool c5 = " << (tt.chanmode5 ? "true" : "false") << "; (void)c5;\n"
      << "  const bool interp = " << (tt.interp ? "true" : "false") << "; (void)interp;\n"
      << "  double *Pw = v.P + tl.fld * 32 + lane; int *Iw = v.I + tl.ints * 32 + lane; (void)Iw;\n"
      << "  double *Vw = v.V + tl.vm * 32 + lane; double *Cw = v.C + tl.pools * 32 + lane; (void)Cw;\n"
      << "  double *Fw = v.F + tl.pools * 32 + lane; double *Gw = v.giv + tl.giv * 32 + lane; (void)Fw; (void)Gw;\n"
      << "  const int64_t neuron = tl.first_neuron + lane; (void)neuron;\n";
    if (mixed) {
        o << "  const float4 *tab = v.tabdf + " << tg.tab_off << "; (void)tab;\n"

          << "  const df xnmin = df_make(" << litf(-tg.xmin_hi) << ", " << litf(-tg.xmin_lo) << "), xinv = df_make("
          << litf(tg.invdx_hi) << ", " << litf(tg.invdx_lo) << "); (void)xnmin; (void)xinv;\n"
          << "  const df ynmin = df_make(" << litf(-tg.ymin_hi) << ", " << litf(-tg.ymin_lo) << "), yinv = df_make("
          << litf(tg.invdy_hi) << ", " << litf(tg.invdy_lo) << "); (void)ynmin; (void)yinv;\n";
    } else {
        o << "  const double *tab = v.tab64 + " << tg.tab_off << "; (void)tab;\n"
          << "  const double *xvals = v.xyvals + " << tg.xv_off << "; (void)xvals;\n"
          << "  const double *yvals = v.xyvals + " << (tg.yv_off >= 0 ? tg.yv_off : tg.xv_off) << "; (void)yvals;\n";
    }
    if (cols)
        o << "  { unsigned dsz; asm(\"mov.u32 %0, %%dynamic_smem_size;\" : \"=r\"(dsz));\n"
          << "    if (dsz < (blockDim.x >> 5) * " << 2 * S * LANES * 8 << "u) { if (v.status) atomicOr(v.status, 4); return; } }\n"
          << "  double *Dc = sm + (size_t)wib * " << 2 * S * LANES << " + lane; double *Rc = Dc + " << S * LANES << ";\n";
    if (!uniform_parent) o << "  const RoRow<int> par{v.parent + tl.topo * 32 + lane};\n";
    // unrolled form of a shared tree: every row is read once per step, so its
    // loads go first out of L1 (measured: mixed 38.6 -> 32.8 us/step on the
    // 16-compartment cables); the looped forms reread rows and keep them
    E.stream = uniform_parent && !cols;
    o << "  const " << (E.stream ? "RoStream" : "RoRow")
      << "<double> Aw{v.A + tl.topo * 32 + lane}, Bw{v.B + tl.topo * 32 + lane}, Cbw{v.Cb + tl.topo * 32 + lane};\n";
    o << "  for (int it = 0; it < nsteps; ++it) {\n"
      << "    const long long step = sbase + step0 + it; (void)step;\n"
      << "    if (v.io_in) {   // this step's inputs into the tile's fields, then visible to every lane\n"
      << "      const double *src = v.io_in + (step - v.io_step0) * v.io_nin; double *Pt = v.P + tl.fld * 32;\n"
      << "      for (int q = v.tin_start[t] + lane; q < v.tin_start[t + 1]; q += 32) {\n"
      << "        const int o = v.tin_off[q]; const double x = src[v.tin_idx[q]];\n"
      << "        if (o & (1 << 30)) { const float hi = __double2float_rn(x); st_df(&Pt[o & ~(1 << 30)], df_make(hi, __double2float_rn(x - (double)hi))); }\n"
      << "        else Pt[o] = x; }\n"
      << "      __syncwarp(); }\n";
    if (mixed) {
        o << "    DCursor vc, cc, c1; vc.row = vc.base = 0; vc.frac = df_make(0.f, 0.f); cc = vc; c1 = vc;\n"
          << "    df Ek = df_make(0.f, 0.f), Gk = Ek, gmax = Ek; (void)gmax;\n";
    } else {
        o << "    VCursor vc, cc;\n";
        if (tg.ncols) o << "    vc.lo = vc.hi = 0.0;\n";
        else o << "    vc.lo = -1e20; vc.hi = 1e20;\n";
        o << "    vc.row = vc.base = 0; vc.frac = 0.0; cc.lo = cc.hi = 0.0; cc.row = cc.base = 0; cc.frac = 0.0;\n"
          << "    double save_frac = 0.0; int tab_base = 0, ctab_base = 0; (void)save_frac; (void)tab_base; (void)ctab_base;\n"
          << "    double Ek = 0.0, Gk = 0.0, gmax = 0.0; (void)gmax;\n";
    }
    o << "    double GHK = 0.0, Ik = 0.0; int doGHK = 0, sel = 0; (void)GHK; (void)doGHK; (void)sel; (void)Ik;\n";
    if (!cols) o << "    double D[" << S << "], R[" << S << "], T[" << S << "]; (void)T;\n";
    else if (uniform_parent) o << "    double T[" << S << "]; (void)T;\n";
    else o << "    double *D = nullptr, *R = nullptr; (void)D; (void)R;\n";
    std::ostringstream save;
    // slot extents in the program
    std::vector<int> sstart(S + 1);
    {
        int off = tt.prog_off;
        for (int s = 0; s < S; ++s) {
            sstart[s] = off;
            for (;;) {
                const int c = prog[off];
                const int n = nops_of(c);
                if (n < 0) return std::string();
                off += 1 + n;
                if (c == M_END) break;
            }
        }
        sstart[S] = off;
    }
    // Static rows of the register form of a shared tree: the rows below the
    // first compartment with channels (TileType::nstatic; programs of
    // M_BEGIN + M_END alone). Their rhs term K = (Em/Rm + inject) * tbyc, D'
    // and T = A / D' change only when a field they come from does, so a
    // launch's first step after such a change (kfull) keeps them -- kst =
    // (K, T), col.y = D' (FP64) or 1/D' (mixed), the stack kernels' layout --
    // and the other steps eliminate only the rhs: R = Vm + K less R_child *
    // T_child, with the arithmetic of the full step (FP64: the same bits).
    // *v.kref: 1, an input writes a static row's Em/Rm, inject or dt/Cm, so K
    // is formed from the fields every step (one pass before the chain); 2, an
    // input writes a diagonal term, so every step is a full one.
    int nst = 0;
    std::vector<std::array<int, 3>> kf;   // per static row: Em/Rm, inject, tbyc fields
    if (uniform_parent && !cols && !giv) {
        nst = std::min(tt.nstatic, S);
        for (int q = 0; q < nst; ++q) {
            const int *a = prog.data() + sstart[q];
            if (sstart[q + 1] - sstart[q] != 9 || a[0] != M_BEGIN || a[5] != M_END) {
                nst = q;
                break;
            }
            kf.push_back({a[1], a[2], a[6]});
        }
    }
    if (nst > 0 && !mixed)   // FP64: the static rows' correctly rounded 1/D' (Markstein's division below)
        o << "  double *kri = v.kri + tl.topo * 32 + lane;\n";
    if (nst > 0)
        o << "  double2 *kst = v.kst + tl.topo * 32 + lane; double2 *col = v.col + tl.topo * 32 + lane;\n"
          << "  const int kr = v.sgen ? *v.kref : 2; const unsigned sgen = v.sgen ? *v.sgen : 0u;\n"
          << "  const bool full = kr > 1 || v.tgen[t] != sgen;\n";
    // K of static row q from its fields, as the slot code forms it
    auto kexpr = [&](int q) {
        const std::string e = std::to_string(kf[q][0] * LANES), i = std::to_string(kf[q][1] * LANES),
                          b = std::to_string(kf[q][2] * LANES);
        if (mixed) return "df_mul(df_add(ld_df_ro(&Pw[" + e + "]), ld_df_cg(&Pw[" + i + "])), ld_df_ro(&Pw[" + b + "]))";
        return "(__ldg(&Pw[" + e + "]) + Pw[" + i + "]) * __ldg(&Pw[" + b + "])";
    };
    std::deque<std::string> pending;   // fused elimination blocks not yet emitted
    const int elim_lag = 1;   // measured: 1 beats 0, 2 and 3 on the 16-compartment cable
    // the channel phase with the fused forward sweep; fast: the static rows
    // from their kept factors
    auto emit_phase = [&](bool fast) -> bool {
    // compact form: runs of four or more identical slot programs become one
    // loop (keeps the kernel inside the instruction cache)
    for (int s = 0; s < S;) {
        std::map<int, int> stride_of;
        const int run = (compact && !giv) ? loop_run(prog, sstart, s, S, stride_of) : 1;
        const int *pc = prog.data() + sstart[s];
        if (run >= 4) {
            E.sidx = "s";
            for (auto &x : stride_of)
                E.fx[x.first] = std::to_string(x.first) + " + " + std::to_string(x.second) + " * (s - " +
                                std::to_string(s) + ")";
            o << "    for (int s = " << s << "; s < " << s + run << "; ++s) {\n";
            if (!emit_slot(E, s, pc, tg)) return false;
            o << "    }\n";
            E.sidx.clear();
            E.fx.clear();
            s += run;
        } else {
            const bool kept = s < nst;
            if (fast && kept) {
                const std::string ks = std::to_string(s * LANES), ss = std::to_string(s);
                o << "    { // slot " << s << ": kept factors\n      const double Vm = Vw[" << ks << "];\n";
                if (mixed) o << "      R[" << ss << "] = df2d(df_add(d2df(Vm), d2df(kst[" << ks << "].x)));\n";
                else o << "      R[" << ss << "] = Vm + kst[" << ks << "].x;\n";
                o << "      D[" << ss << "] = col[" << ks << "].y; T[" << ss << "] = kst[" << ks << "].y;";
                if (!mixed) o << " Y[" << ss << "] = kri[" << ks << "];";
                o << " }\n";
            } else if (!emit_slot(E, s, pc, tg)) {
                return false;
            }
            if (uniform_parent) {
                // forward elimination fused into the channel phase: row s pulls
                // its children (ascending, the order the separate sweep pushes
                // them in, so the arithmetic is unchanged) and prepares its own
                // factor for its parent. It is emitted after the channel code
                // of the next `lag` compartments, so that its chain of FP64
                // operations overlaps their loads and FP32 arithmetic
                const std::vector<int> &par = *uniform_parent;
                std::ostringstream el;
                el << "    {";
                for (int c = 0; c < s && fast && kept; ++c) {   // a kept row: the rhs only
                    if (par[c] != s) continue;
                    if (mixed) el << " R[" << s << "] = fma(-R[" << c << "], T[" << c << "], R[" << s << "]);";
                    else el << " R[" << s << "] -= R[" << c << "] * T[" << c << "];";
                }
                for (int c = 0; c < s && !(fast && kept); ++c) {
                    if (par[c] != s) continue;
                    if (mixed)
                        el << " D[" << s << "] = fma(-Bw[" << c * LANES << "], T[" << c << "], D[" << s << "]); R[" << s
                           << "] = fma(-R[" << c << "], T[" << c << "], R[" << s << "]);";
                    else
                        el << " D[" << s << "] -= Bw[" << c * LANES << "] * T[" << c << "]; R[" << s << "] -= R[" << c
                           << "] * T[" << c << "];";
                }
                if (fast && kept) {
                } else if (mixed) {
                    el << " const double ri = rcp_newton(D[" << s << "]); D[" << s << "] = ri;";
                    if (par[s] >= 0) el << " T[" << s << "] = Aw[" << s * LANES << "] * ri;";
                } else {
                    // FP64: one correctly rounded y = 1/D' per row; T = A/D' and the back
                    // substitution's quotient by Markstein's correction (the divisions' bits)
                    el << " Y[" << s << "] = 1.0 / D[" << s << "];";
                    if (par[s] >= 0)
                        el << " { const double a = Aw[" << s * LANES << "], qa = a * Y[" << s << "]; T[" << s
                           << "] = fma(fma(-D[" << s << "], qa, a), Y[" << s << "], qa); }";
                }
                if (!fast && kept) {   // keep K, T and D' (1/D')
                    const std::string ks = std::to_string(s * LANES);
                    el << "\n      if (full) {";
                    if (mixed) el << " kst[" << ks << "].x = df2d(" << kexpr(s) << ");";
                    else el << " kst[" << ks << "].x = " << kexpr(s) << ";";
                    el << " kst[" << ks << "].y = " << (par[s] >= 0 ? "T[" + std::to_string(s) + "]" : std::string("0.0"))
                       << "; col[" << ks << "].y = D[" << s << "]; }";
                    if (!mixed) el << " kri[" << ks << "] = Y[" << s << "];";
                }
                el << " }\n";
                pending.push_back(el.str());
                if ((int)pending.size() > elim_lag) {
                    o << pending.front();
                    pending.pop_front();
                }
            }
            ++s;
        }
    }
    for (const std::string &x : pending) o << x;
    pending.clear();
    return true;
    };
    if (uniform_parent && !mixed) o << "    double Y[" << S << "];\n";   // FP64: each row's 1/D'
    if (nst > 0) {
        o << "    const bool kfull = full && (it == 0 || kr > 1);\n    if (kfull) {\n";
        if (!emit_phase(false)) return std::string();
        o << "    } else {\n";
        // inputs on the static rows' rhs fields: this step's K of every
        // static row from its fields, before the chain (not inside it)
        o << "    if (kr) {";
        for (int q = 0; q < nst; ++q)
            o << " kst[" << q * LANES << "].x = " << (mixed ? "df2d(" + kexpr(q) + ")" : kexpr(q)) << ";";
        o << " }\n";
        if (!emit_phase(true)) return std::string();
        o << "    }\n";
    } else if (!emit_phase(false)) {
        return std::string();
    }
    std::string body = o.str();
    if (cols) {
        // rewrite D[s]/R[s] into the shared columns
        std::string out;
        out.reserve(body.size());
        for (size_t i = 0; i < body.size(); ++i) {
            if ((body[i] == 'D' || body[i] == 'R') && i + 1 < body.size() && body[i + 1] == '[' &&
                (i == 0 || !(isalnum((unsigned char)body[i - 1]) || body[i - 1] == '_'))) {
                size_t j = body.find(']', i);
                const std::string idx = body.substr(i + 2, j - i - 2);
                out += (body[i] == 'D' ? "Dc[(" : "Rc[(") + idx + ") * 32]";
                i = j;
            } else {
                out += body[i];
            }
        }
        body = out;
    }
    std::ostringstream t;
    t << body;
    // pools
    const int *pp = prog.data() + tt.pool_off;
    while (pp[0] != 0) {
        if (pp[0] != PO_CACONC) return std::string();
        t << "    { double *cx = &Cw[" << pp[1] * LANES << "]; const double base = Pw[" << pp[2] * LANES
          << "]; const double itau = Pw[" << pp[3] * LANES << "];\n"
          << "      *cx = base + ((*cx - base) * (2.0 - itau) + (Fw[" << pp[1] * LANES << "] * Pw[" << pp[4] * LANES
          << "])) / itau; }\n";
        pp += 5;
    }
    // elimination
    auto Dx = [&](int s) { return !cols ? "D[" + std::to_string(s) + "]" : "Dc[" + std::to_string(s * LANES) + "]"; };
    auto Rx = [&](int s) { return !cols ? "R[" + std::to_string(s) + "]" : "Rc[" + std::to_string(s * LANES) + "]"; };
    if (uniform_parent) {
        const std::vector<int> &par = *uniform_parent;   // forward sweep already fused above
        for (int s = S - 1; s >= 0; --s) {
            const int p = par[s];
            t << "    { double r = " << Rx(s) << ";";
            if (p >= 0) {
                if (mixed) t << " r = fma(-Cbw[" << s * LANES << "], " << Rx(p) << ", r);";
                else t << " r -= Cbw[" << s * LANES << "] * " << Rx(p) << ";";
            }
            if (mixed) {
                t << " r = r * " << Dx(s) << ";";
            } else {
                // RN(r / D') from the correctly rounded y = 1/D' by Markstein's
                // correction, the division's bits (one DMUL, two DFMAs)
                t << " { const double q = r * Y[" << s << "]; r = fma(fma(-" << Dx(s) << ", q, r), Y[" << s << "], q); }";
            }
            t << " " << Rx(s) << " = r;";
            if (tt.crank) {
                if (mixed) t << " Vw[" << s * LANES << "] = fma(2.0, r, -Vw[" << s * LANES << "]);";
                else t << " Vw[" << s * LANES << "] = r + r - Vw[" << s * LANES << "];";
            } else {
                t << " Vw[" << s * LANES << "] = r;";
            }
            t << " }\n";
        }
    } else {
        t << "    for (int s = 0; s < " << S << "; ++s) { const int p = par[s * 32];\n";
        if (mixed)
            t << "      const double ri = rcp_newton(Dc[s * 32]); Dc[s * 32] = ri;\n"
              << "      if (p >= 0) { const double temp = Aw[s * 32] * ri; Dc[p * 32] = fma(-Bw[s * 32], temp, Dc[p * 32]); Rc[p * 32] = fma(-Rc[s * 32], temp, Rc[p * 32]); } }\n";
        else
            t << "      if (p >= 0) { const double d = Dc[s * 32]; const double temp = Aw[s * 32] / d; Dc[p * 32] -= Bw[s * 32] * temp; Rc[p * 32] -= Rc[s * 32] * temp; } }\n";
        t << "    for (int s = " << S - 1 << "; s >= 0; --s) { const int p = par[s * 32]; double r = Rc[s * 32];\n";
        if (mixed) t << "      if (p >= 0) r = fma(-Cbw[s * 32], Rc[p * 32], r); r = r * Dc[s * 32];\n";
        else t << "      if (p >= 0) r -= Cbw[s * 32] * Rc[p * 32]; r = r / Dc[s * 32];\n";
        t << "      Rc[s * 32] = r;";
        if (tt.crank) {
            if (mixed) t << " Vw[s * 32] = fma(2.0, r, -Vw[s * 32]);";
            else t << " Vw[s * 32] = r + r - Vw[s * 32];";
        } else {
            t << " Vw[s * 32] = r;";
        }
        t << " }\n";
    }
    t << "    finite_check(v, Vw[0], active);\n";
    if (nst > 0) t << "    if (kfull && it == 0) { __syncwarp(); if (lane == 0) v.tgen[t] = sgen; }\n";
    t << "    if (v.io_out) {   // this step's outputs\n"
      << "      __syncwarp(); double *dst = v.io_out + (step - v.io_step0) * v.io_nout; const double *Vt = v.V + tl.vm * 32;\n"
      << "      for (int q = v.tout_start[t] + lane; q < v.tout_start[t + 1]; q += 32) dst[v.tout_idx[q]] = Vt[v.tout_off[q]]; }\n";
    t << "  }\n}\n";
    return t.str();
}

bool jit_available(std::string *why)
{
    std::call_once(g_api_once, init_api);
    if (!g_api.ok && why) *why = g_api.why;
    return g_api.ok;
}

int jit_compile(const std::string &src, bool fp64_exact, int device_major, int device_minor, JitKernel *out,
                std::string *log)
{
    if (!jit_available(log)) return -1;
    nvrtcProgram prog;
    const char *hdr_src[] = {kSrc_gbh_internal_h, kSrc_gbh_df_cuh, kSrc_gbh_devfn_cuh, "", kStdintStub};
    const char *hdr_name[] = {"gbh_internal.h", "gbh_df.cuh", "gbh_devfn.cuh", "cuda_runtime.h", "stdint.h"};
    if (g_api.create(&prog, src.c_str(), "gbh_jit.cu", 5, hdr_src, hdr_name) != NVRTC_SUCCESS) {
        if (log) *log = "nvrtcCreateProgram failed";
        return -1;
    }
    char arch[64];
    snprintf(arch, sizeof(arch), "--gpu-architecture=sm_%d%da", device_major, device_minor);
    std::vector<const char *> opts = {arch, "--std=c++17", "-default-device", "-lineinfo"};
    if (fp64_exact) opts.push_back("--fmad=false");
    const nvrtcResult rc = g_api.compile(prog, (int)opts.size(), opts.data());
    size_t ls = 0;
    g_api.logsize(prog, &ls);
    if (log && ls > 1) {
        log->resize(ls);
        g_api.getlog(prog, &(*log)[0]);
    }
    if (rc != NVRTC_SUCCESS) {
        g_api.destroy(&prog);
        return -1;
    }
    size_t cs = 0;
    g_api.cubinsize(prog, &cs);
    std::vector<char> cubin(cs);
    g_api.getcubin(prog, cubin.data());
    g_api.destroy(&prog);
    CUmodule mod;
    if (g_api.load(&mod, cubin.data()) != CUDA_SUCCESS) {
        if (log) *log += "\ncuModuleLoadData failed";
        return -1;
    }
    CUfunction fn;
    if (g_api.getfn(&fn, mod, "gbh_jit") != CUDA_SUCCESS) {
        g_api.unload(mod);
        if (log) *log += "\ncuModuleGetFunction failed";
        return -1;
    }
    out->module = mod;
    out->fn = fn;
    return 0;
}

cudaError_t jit_launch(const JitKernel &k, const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                       long long step, size_t smem, cudaStream_t st)
{
    const int ntiles = tile1 - tile0;
    const int blocks = (ntiles + warps - 1) / warps;
    if (smem > 48 * 1024) {
        if (g_api.setattr((CUfunction)k.fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem) != CUDA_SUCCESS)
            return cudaErrorLaunchFailure;
    }
    DevView vv = v;
    void *args[] = {&vv, &tile0, &tile1, &smax, &nsteps, &step};
    const CUresult r = g_api.launch((CUfunction)k.fn, blocks, 1, 1, warps * LANES, 1, 1, (unsigned)smem,
                                    (CUstream)st, args, nullptr);
    if (r == CUDA_SUCCESS) return cudaSuccess;
    // a fault of earlier work stays a launch failure; a launch this device
    // refuses (resources, shared memory) is a configuration error
    return r == CUDA_ERROR_LAUNCH_FAILED || r == CUDA_ERROR_ILLEGAL_ADDRESS ? cudaErrorLaunchFailure
                                                                          : cudaErrorInvalidConfiguration;
}

void jit_release(JitKernel &k)
{
    if (k.module && g_api.ok) g_api.unload((CUmodule)k.module);
    k.module = nullptr;
    k.fn = nullptr;
}

}  // namespace gbh
