/*
 * hsolve_oracle.c -- CPU restatement of the GENESIS hsolve chanmode 4/5 step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle). See hsolve_oracle.h for the mapping
 * of each function to the reference source it restates. The control flow is
 * written as an explicit cursor machine over ops[]/chip[]/givals[]; every
 * arithmetic expression keeps the reference's operand order so that, built
 * with -ffp-contract=off, results are bit-identical to the reference step.
 */
#include "hsolve_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* opcode values, genesis/src/hines/hines_defs.h:178-222 */
enum {
    OP_TABCURR = 0, OP_COMPT = 100, OP_FCOMPT = 101, OP_LCOMPT = 102,
    OP_SPIKE = 200, OP_ELMMPUMP = 500, OP_CONC_VAL = 1000, OP_NERNST = 2000,
    OP_GHK = 2010, OP_CHAN = 3000, OP_CHAN_EK = 3001, OP_SAME_GHK = 3002,
    OP_DO_TABGHK = 3003, OP_ADD_CURR = 3200, OP_FLUX = 3300, OP_SCALE_FLUX = 3301,
    OP_STORE_ALLI = 3501, OP_STORE_ALLC = 3502, OP_IPOL1V = 4001, OP_IPOL1C = 4002,
    OP_IPOL2V = 4003, OP_IPOL2C = 4004, OP_SYN2 = 4100, OP_SYN3 = 4101,
    OP_MGBLOCK = 4200, OP_NEWVOLT = 5100, OP_NEWCONC1 = 5110, OP_NEWCONC2 = 5111,
    OP_DOMAIN = 5112,
    /* concops */
    CO_CONC = 10100, CO_FCONC = 10101, CO_LCONC = 10102, CO_FLUXCONC = 10103,
    CO_CACONC = 10200, CO_LCACONC = 10202, CO_TAUPUMP = 11000, CO_CTAUPUMP = 11001,
    CO_MMPUMP = 11010, CO_HILLPUMP = 11011, CO_PHILLPUMP = 11012, CO_BUFFER = 12000,
    CO_POOL = 12100
};
/* funcs codes, hines_defs.h:120-128 */
enum { F_ELIM = 0, F_SET_DIAG = 1, F_SKIP_DIAG = 2, F_FASTSIB = 3, F_COPY = 4,
       F_SIB = 5, F_CALC = 6, F_FINISH = 7 };

#define ORC_TINY 1.0e-6 /* hines_defs.h TINY */

/* SYN3_OP's uniform deviate, urandom() = G_RNG() in the reference: with its
 * default generator selected (sim/sim_random.c:45-100, 197-210) that is
 * "ran1" of Numerical Recipes in C (Press et al., 1st ed., sec. 7.1): three
 * linear congruential generators; the first two make a value in [0, 1),
 * the third picks which of 97 stored values to return and to replace with
 * the new one. Restated here with the published constants; values are
 * stored and returned as float, as G_RNG returns them. One stream for the
 * process, (re)seeded by orc_seed_rng (G_SEEDRNG's ran1(-seed)); unseeded,
 * it starts as ran1(0) does on its first call. */
enum { R1_M1 = 259200, R1_A1 = 7141, R1_C1 = 54773, R1_M2 = 134456, R1_A2 = 8121, R1_C2 = 28411,
       R1_M3 = 243000, R1_A3 = 4561, R1_C3 = 51349 };
static struct {
    long x1, x2, x3;
    float tab[98];
    int ready;
} orc_rng;

/* a generated value: (x1 + x2 / M2) / M1, evaluated in that order (the
 * reference's constants RM1, RM2 are unparenthesised (1.0)/M quotients) */
static float orc_ran1_value(void)
{
    return (float)(((double)orc_rng.x1 + (double)orc_rng.x2 / R1_M2) / R1_M1);
}

static void orc_ran1_init(long seed)
{
    int j;
    orc_rng.x1 = (R1_C1 + seed) % R1_M1;
    orc_rng.x1 = (R1_A1 * orc_rng.x1 + R1_C1) % R1_M1;
    orc_rng.x2 = orc_rng.x1 % R1_M2;
    orc_rng.x1 = (R1_A1 * orc_rng.x1 + R1_C1) % R1_M1;
    orc_rng.x3 = orc_rng.x1 % R1_M3;
    for (j = 1; j <= 97; j++) {
        orc_rng.x1 = (R1_A1 * orc_rng.x1 + R1_C1) % R1_M1;
        orc_rng.x2 = (R1_A2 * orc_rng.x2 + R1_C2) % R1_M2;
        orc_rng.tab[j] = orc_ran1_value();
    }
    orc_rng.ready = 1;
}

static double orc_urandom(void)
{
    int j;
    float out;
    if (!orc_rng.ready) orc_ran1_init(0);
    orc_rng.x1 = (R1_A1 * orc_rng.x1 + R1_C1) % R1_M1;
    orc_rng.x2 = (R1_A2 * orc_rng.x2 + R1_C2) % R1_M2;
    orc_rng.x3 = (R1_A3 * orc_rng.x3 + R1_C3) % R1_M3;
    j = 1 + (int)((97 * orc_rng.x3) / R1_M3);
    out = orc_rng.tab[j];
    orc_rng.tab[j] = orc_ran1_value();
    return (double)out;
}

/* G_SEEDRNG(seed): ran1(-seed), which reinitialises and then draws once */
void orc_seed_rng(long seed)
{
    orc_ran1_init(seed);
    (void)orc_urandom();
}

/*
 * Table-lookup cursor shared by all compartments of one call: the reference
 * keeps the last bracket (xlo, xhi, row) and only recomputes the row when Vm
 * leaves it (hines_chip.c:174-203, 236-262).
 */
typedef struct {
    double lo, hi;  /* bracket of the cached row                         */
    int row;        /* cached row index                                  */
    double frac;    /* interpolation fraction inside the row             */
    int base;       /* tablist offset of the cached row (row*ncols)      */
} orc_cursor;

static void orc_locate(orc_cursor *c, double v, double vmin, double inv, int divs,
                       const double *vals, int ncols, int interpolate)
{
    if (interpolate) {
        double f = (v - vmin) * inv;
        if ((c->lo > v) || (v >= c->hi)) {
            if (f < 0.0)
                f = 0.0;
            else if (f > divs)
                f = divs;
            c->row = (int)f;
            f = f - (double)c->row;
            c->lo = vals[c->row];
            c->hi = vals[c->row + 1];
            c->base = c->row * ncols;
        } else {
            f = f - (double)c->row;
        }
        c->frac = f;
    } else {
        /* calcmode 0: nearest lower row, no fraction (hines_chip.c:192-201) */
        if ((c->lo > v) || (v >= c->hi)) {
            int k = (int)((v - vmin) * inv);
            if (k < 0)
                k = 0;
            else if (k > divs)
                k = divs;
            c->row = k;
            c->lo = vals[k];
            c->hi = vals[k + 1];
            c->base = k * ncols;
        }
        c->frac = 0.0;
    }
}

/* Raise a gate value to an integer power with the reference's multiply order
 * (hines_chip.c:490-509) and scale the running conductance. */
static double orc_power(double g, double x, int p)
{
    switch (p) {
    case 1: return g * x;
    case 2: return g * (x * x);
    case 3: return g * (x * x * x);
    case 4: x *= x; return g * (x * x);
    case 5: g *= x; x *= x; x *= x; return g * x;
    default: x *= x; g *= x; x *= x; return g * x; /* 6 */
    }
}

int orc_chip_update(orc_solver *s)
{
    const int interp = s->calcmode != 0;
    const int chanmode5 = (s->chanmode == 5);
    const int storeall = s->storemode;
    const int ncols = s->ncols;
    int *ops = s->ops;
    double *chip = s->chip;
    double *results = s->results;
    double *givals = s->givals + 1;
    const double *tablist = s->tablist;
    const double *stablist = s->stablist;
    int o = 0, c = 0, g = 0, row = 0;
    orc_cursor vc, cc;
    double vipol_saved = 0.0;      /* 'ipol' of NEWCONC2 (hines_chip.c:224-232) */
    int ctab_base = 0, tab_base = 0;
    int concin = 0;                /* index into conc/flux (CONC_VAL_OP)        */
    double Ek = 0.0, Gk = 0.0, gmax = 0.0, Ik = 0.0, GHK = 0.0;
    int doGHK = 0;

    if (tablist) {
        vc.lo = vc.hi = 0.0;
    } else { /* passive model: the bracket never needs recomputing */
        vc.lo = -1e20;
        vc.hi = 1e20;
    }
    vc.row = 0; vc.frac = 0.0; vc.base = 0;
    cc.lo = cc.hi = 0.0; cc.row = 0; cc.frac = 0.0; cc.base = 0;
    if (storeall && s->itotal) {
        int k;
        for (k = 0; k < s->nelm_names; k++) s->itotal[k] = 0.0;
    }

    /* one iteration per compartment; ops[o] is FCOMPT/COMPT/LCOMPT */
    while (ops[o++] != OP_LCOMPT) {
        const double Vm = s->vm[row];
        double sumg = 0.0;
        double ichan = chip[c] + chip[c + 1];       /* Em/Rm + inject */
        double Im = chip[c] - Vm / givals[g];       /* leak: Em/Rm - Vm/Rm */
        g++;
        givals[g++] = Im;
        if (storeall == 1) s->itotal[0] += Im;
        c += 2;

        while (ops[o] > OP_LCOMPT) {
            const int code = ops[o++];
            int current = 0; /* 1: fall through to the conductance loop */
            double X, Y;
            switch (code) {
            case OP_NEWVOLT:
                orc_locate(&vc, Vm, s->xmin, s->invdx, s->xdivs, s->xvals, ncols, interp);
                continue;
            case OP_CONC_VAL:
                concin = ops[o++];
                s->flux[concin] = 0.0;
                continue;
            case OP_DOMAIN: {
                double concen = chip[c++] * Ik;
                orc_locate(&cc, concen, s->ymin, s->invdy, s->ydivs, s->yvals, ncols, interp);
                ctab_base = cc.base;
                continue;
            }
            case OP_NEWCONC2: {
                double concen = s->conc[ops[o++]];
                tab_base = ctab_base;       /* keep the C1 position */
                vipol_saved = cc.frac;
                orc_locate(&cc, concen, s->ymin, s->invdy, s->ydivs, s->yvals, ncols, interp);
                ctab_base = cc.base;
                continue;
            }
            case OP_NEWCONC1: {
                double concen = s->conc[concin];
                orc_locate(&cc, concen, s->ymin, s->invdy, s->ydivs, s->yvals, ncols, interp);
                ctab_base = cc.base;
                continue;
            }
            case OP_SPIKE:
                ops[o] -= 1; /* refractory countdown */
                if (Vm > chip[c++]) {
                    if (ops[o] <= 0) {
                        if (s->on_spike) s->on_spike(s->hook_ctx, s->id);
                        ops[o] = ops[o + 1];
                    }
                }
                o += 2;
                continue;
            case OP_ELMMPUMP: {
                double *cx = &s->conc[concin];
                X = 1.0 / (*cx + chip[c++]);
                ichan += Ik = chip[c] * *cx * X;
                if (chanmode5) {
                    givals[g++] = Ik / chip[c++];
                } else {
                    givals[g++] = Ik;
                    c++;
                }
                Im += Ik;
                s->codiag[concin] += chip[c++] * X;
                continue;
            }
            case OP_FLUX:
                s->flux[concin] += Ik;
                continue;
            case OP_STORE_ALLI:
                s->itotal[ops[o++]] += Ik;
                continue;
            case OP_STORE_ALLC:
                s->itotal[ops[o++]] += Gk;
                continue;
            case OP_SCALE_FLUX:
                s->flux[concin] += chip[c++] * Ik;
                continue;
            case OP_GHK: {
                const double cin = s->conc[concin], cout = s->conc[concin + 1];
                GHK = chip[c++];               /* zF/RT */
                X = Vm * GHK;
                Y = exp(-X);
                Ek = chip[c++];                /* zF */
                Ik = Ek * (cin - (Y * cout));
                if (fabs(X) < ORC_TINY) {
                    Gk = 1.0 - 0.5 * X;
                    GHK = 0.5 * GHK * Ek * (cin + cout);
                    Ik = -Ik / Gk;
                } else {
                    Gk = 1.0 - Y;
                    GHK = GHK * (Ik / Gk - Ek * GHK * (cin - cout) * Vm * Y / (Gk * Gk));
                    Ik = -X * Ik / Gk;
                }
                Ek = (Ik + GHK * Vm) / GHK;
                gmax = chip[c++];
                Gk = gmax * GHK;
                current = 1;
                break;
            }
            case OP_SAME_GHK:
                gmax = chip[c++];
                Gk = gmax * GHK;
                current = 1;
                break;
            case OP_DO_TABGHK:
                doGHK = 1;
                current = 1;
                break;
            case OP_NERNST:
                Ek = log(s->conc[concin + 1] / s->conc[concin]) * chip[c++];
                gmax = Gk = chip[c++];
                current = 1;
                break;
            case OP_CHAN_EK:
                Ek = chip[c++];
                gmax = Gk = chip[c++];
                current = 1;
                break;
            case OP_CHAN:
                gmax = Gk = chip[c++];
                current = 1;
                break;
            default:
                s->err_op = o - 1;
                return -1;
            }
            if (!current) continue;

            /* conductance sub-program until the current is added */
            for (;;) {
                int k = ops[o++];
                int gate = 0; /* 1: X (B') and Y (A') are ready for DOPOWER */
                if (k == OP_IPOL1V) {
                    const int b = vc.base + ops[o++];
                    if (interp) {
                        X = tablist[b];
                        X = X + vc.frac * (tablist[b + ncols] - X);
                        Y = tablist[b + 1];
                        Y = Y + vc.frac * (tablist[b + 1 + ncols] - Y);
                    } else {
                        X = tablist[b];
                        Y = tablist[b + 1];
                    }
                    tab_base = b + 1; /* the reference's tab ends one past the B' entry */
                    gate = 1;
                } else if (k == OP_IPOL1C) {
                    const int b = ctab_base + ops[o++];
                    if (interp) {
                        X = tablist[b];
                        X = X + cc.frac * (tablist[b + ncols] - X);
                        Y = tablist[b + 1];
                        Y = Y + cc.frac * (tablist[b + 1 + ncols] - Y);
                    } else {
                        X = tablist[b];
                        Y = tablist[b + 1];
                    }
                    tab_base = b + 1; /* the reference's tab ends one past the B' entry */
                    gate = 1;
                } else if (k == OP_IPOL2V || k == OP_IPOL2C) {
                    const double rf = (k == OP_IPOL2V) ? vc.frac : vipol_saved;
                    const int b = ((k == OP_IPOL2V) ? vc.base : tab_base) + cc.row + cc.row + ops[o++];
                    if (interp) {
                        const int n = b + ncols;
                        X = (1.0 - rf) * ((1.0 - cc.frac) * tablist[b] + cc.frac * tablist[b + 2]) +
                            rf * ((1.0 - cc.frac) * tablist[n] + cc.frac * tablist[n + 2]);
                        Y = (1.0 - rf) * ((1.0 - cc.frac) * tablist[b + 1] + cc.frac * tablist[b + 3]) +
                            rf * ((1.0 - cc.frac) * tablist[n + 1] + cc.frac * tablist[n + 3]);
                    } else {
                        X = tablist[b];
                        Y = tablist[b + 1];
                    }
                    tab_base = b + 1; /* the reference's tab ends one past the B' entry */
                    gate = 1;
                } else if (k >= OP_SYN2) {
                    int stab;
                    if (k == OP_SYN3) {
                        if (orc_urandom() <= chip[c++]) chip[c] += stablist[ops[o] + 3];
                    }
                    stab = ops[o++];
                    chip[c] *= stablist[stab]; /* X*xconst2 */
                    if (ops[o] == 0) {
                        if (s->on_syn)
                            ops[o] = s->on_syn(s->hook_ctx, s->id, stab, ops[o + 1], c);
                        else
                            ops[o] = -1;
                    }
                    ops[o] -= 1;
                    o += 2;
                    X = chip[c++];
                    chip[c] = X * stablist[stab + 1] + chip[c] * stablist[stab + 2];
                    Gk *= chip[c++];
                    if (ops[o] == OP_MGBLOCK) {
                        if (chanmode5) {
                            givals[g++] = Gk / gmax;
                            givals[g++] = Gk * (Ek - Vm) / gmax;
                        } else {
                            givals[g++] = Gk;
                            givals[g++] = Gk * (Ek - Vm);
                        }
                        givals[g++] = Ek;
                        X = chip[c] * exp(Vm * chip[c + 1]);
                        c += 2;
                        Gk *= X / (X + chip[c++]);
                        o++;
                    }
                    k = OP_ADD_CURR;
                } else if (k != OP_ADD_CURR) {
                    s->err_op = o - 1;
                    return -1;
                }

                if (gate) {
                    const int p = ops[o++];
                    if (p == 0) { /* tabcurrent or GHK tabcurrent */
                        Ek = Y;
                        if (doGHK) {
                            GHK = X;
                            doGHK = 0;
                            break; /* no current computed here */
                        }
                        Gk *= X;
                        k = OP_ADD_CURR;
                    } else {
                        int pw = p;
                        if (p > 0) {
                            X = chip[c] = (chip[c] * (2.0 - X) + Y) / X;
                        } else {       /* instantaneous gate */
                            X = chip[c] = Y / X;
                            pw = -p;
                        }
                        c++;
                        Gk = orc_power(Gk, X, pw);
                        continue;
                    }
                }
                if (k == OP_ADD_CURR) {
                    sumg += Gk;
                    ichan += Ek * Gk;
                    if (chanmode5) {
                        givals[g++] = Gk / gmax;
                        Ik = Gk * (Ek - Vm);
                        givals[g++] = Ik / gmax;
                    } else {
                        givals[g++] = Gk;
                        givals[g++] = Ik = Gk * (Ek - Vm);
                    }
                    givals[g++] = Ek;
                    Im += Ik;
                    break;
                }
            }
        }
        /* store this compartment's row: chip[c]=tbyc, chip[c+1]=diagterm */
        results[2 * row] = Vm + ichan * chip[c];
        results[2 * row + 1] = sumg * chip[c] + chip[c + 1];
        c += 2;
        givals[g++] = Im;
        row++;
    }
    return 0;
}

int orc_conc_update(orc_solver *s)
{
    int *op = s->concops;
    double *chip = s->concchip;
    double *conc = s->conc, *flux = s->flux, *codiag = s->codiag, *coresult = s->coresult;
    double *ov = s->ovals;
    const double dt = s->dt;
    int index = 0;
    double result = 0.0;
    int o = 0, c = 0;
    if (!op) return 0;
    for (;;) {
        switch (op[o++]) {
        case CO_CONC:
            coresult[index] = result;
            /* fall through */
        case CO_FCONC:
            index = op[o++];
            result = 0.0;
            break;
        case CO_FLUXCONC:
            result += chip[c] + flux[index] * chip[c + 1];
            c += 2;
            break;
        case CO_CTAUPUMP:
            result += chip[c++];
            codiag[index] += chip[c++];
            break;
        case CO_TAUPUMP: {
            double itau = dt / (chip[c] + chip[c + 1] *
                                (exp((s->vm[op[o++]] - chip[c + 2]) * chip[c + 3])));
            if (ov) *ov++ = itau;
            c += 4;
            result += chip[c++] * itau;
            codiag[index] += itau;
            break;
        }
        case CO_MMPUMP:
            codiag[index] += chip[c] / (conc[index] + chip[c + 1]);
            c += 2;
            break;
        case CO_HILLPUMP: {
            double X = conc[index], h;
            int k = op[o++];
            h = (k == 2) ? X : (k == 3) ? X * X : (k == 4) ? X * X * X : 1.0;
            h = h / (h * X + chip[c++]);
            codiag[index] += chip[c++] * h;
            break;
        }
        case CO_PHILLPUMP: {
            int k = op[o++];
            double X = conc[op[o]], h;
            h = (k == 2) ? X : (k == 3) ? X * X : (k == 4) ? X * X * X : 1.0;
            h = h / (h * X + chip[c++]);
            codiag[op[o++]] += chip[c++] * h;
            result += chip[c++] * h * X;
            break;
        }
        case CO_LCONC:
            coresult[index] = result;
            return 0;
        case CO_BUFFER: {
            double *bf = &conc[op[o++]];
            double X = chip[c++], b;
            b = ((1.0 - X) * *bf + chip[c]) / (1.0 + X + chip[c + 1] * conc[index]);
            result += b - *bf;
            *bf = b;
            c += 2;
            break;
        }
        case CO_POOL:
            conc[index] += result;
            break;
        case CO_CACONC: {
            const int k = op[o++];
            const double base = chip[c++];
            const double itau = chip[c++];
            conc[k] = base + ((conc[k] - base) * (2.0 - itau) + (flux[k] * chip[c++])) / itau;
            break;
        }
        case CO_LCACONC:
            return 0;
        default:
            return -1;
        }
    }
}

/*
 * Concentration diffusion (difshell systems), do_h_conc_solve
 * (hines_conc.c:39-396). Each system i holds nshells[i] shells of
 * nshrows[i] rows: nshfix[i] fixed buffers, then diffusible buffers, then the
 * shell's free concentration, at conc[dconc[i] + shell*rows + row]. covals0
 * is consumed in order across the systems; codiag/coresult carry what the
 * pumps and fluxes of the concops program added this step, and codiag is
 * reset to 1 once used. Crank-Nicolson systems without buffers return
 * 2x - c (hines_conc.c:380-387); the buffered form is written for either
 * method (setup scales its terms by dt or dt/2).
 */

/* Shells only: tridiagonal in the shell index (hines_conc.c:337-395). */
static void diff_shells(orc_solver *s, int c0, int ms, int *cursor)
{
    double *conc = s->conc, *cd = s->codiag, *cr = s->coresult;
    double *fac = s->covals, *part = s->cores;
    const double *k = s->covals0;
    int q = *cursor, m, c = c0;
    double up = k[q++], dn, d, f, x;
    d = up + cd[c];
    cd[c] = 1.0;
    part[0] = (conc[c] + cr[c]) / d;
    for (m = 1; m < ms - 1; m++) {
        f = fac[m] = -up / d;
        dn = k[q];
        up = k[q + 1];
        q += 2;
        c++;
        d = cd[c] + dn * (1.0 + f) + up;
        cd[c] = 1.0;
        part[m] = (conc[c] + cr[c] + dn * part[m - 1]) / d;
    }
    f = fac[m] = -up / d;
    dn = k[q++];
    c++;
    d = cd[c] + dn * (1.0 + f);
    cd[c] = 1.0;
    x = (conc[c] + cr[c] + dn * part[m - 1]) / d;
    if (s->crank) {
        conc[c] = x + x - conc[c];
        for (m--, c--; m >= 0; m--, c--) {
            x = part[m] - fac[m + 1] * x;
            conc[c] = x + x - conc[c];
        }
    } else {
        conc[c] = x;
        for (m--, c--; m >= 0; m--, c--) {
            x = part[m] - fac[m + 1] * x;
            conc[c] = x;
        }
    }
    *cursor = q;
}

/* Shells with buffers: banded system, rows of a shell eliminated as they are
 * filled (hines_conc.c:123-335). Scratch layout: fac[(shell*rows + row)*rows
 * + column], part[shell*rows + row]. */
static void diff_buffered(orc_solver *s, int c0, int ms, int w, int nfix, int b0, int *cursor)
{
    double *conc = s->conc, *cd = s->codiag, *cr = s->coresult;
    double *fac = s->covals, *part = s->cores;
    const double *k = s->covals0, *bv = s->bufvals;
    const int w1 = w - 1, sq = w * w, last = ms - 1;
    int q = *cursor, m, n, nb, nc = c0, pr = 0, prev_shell = -1;
    int row = 0, srow = sq - w, srow_prev = srow - sq, cs = c0 + w1;
    double co = conc[cs], dsh, rsh, d, t, t2, h;

    for (m = 0; m < ms; m++) {
        dsh = cd[cs];
        cd[cs] = 1.0;
        rsh = cr[cs];
        /* fixed buffers: no coupling to other shells */
        for (n = 0, nb = b0; n < nfix; n++, nb += 3) {
            fac[srow + n] = d = bv[nb] * co + bv[nb + 1];
            dsh += t = bv[nb] * conc[nc];
            d = 1.0 / (1.0 + d);
            fac[row] = t * d;
            rsh += t2 = -bv[nb + 1] * conc[nc] + k[q++];
            part[pr++] = (conc[nc] + t2) * d;
            nc++;
            row += w;
        }
        /* diffusible buffers: coupled to the same buffer in the neighbours */
        for (; n < w1; n++, nb += 3) {
            fac[srow + n] = d = bv[nb] * co + bv[nb + 1];
            dsh += t = bv[nb] * conc[nc];
            rsh += t2 = -bv[nb + 1] * conc[nc] + bv[nb + 2];
            if (m) {
                h = k[q] * fac[row - sq];
                if (m < last) {
                    d += 1.0 + k[q + 1] + k[q] * (1.0 + fac[row - sq + 1]) - h * fac[srow_prev + n];
                    fac[row + 1] = -k[q + 1] / d;
                    t2 += k[q] * conc[nc - w] + (1.0 - k[q] - k[q + 1]) * conc[nc] + k[q + 1] * conc[nc + w];
                } else {
                    d += 1.0 + k[q] * (1.0 + fac[row - sq + 1]) - h * fac[srow_prev + n];
                    t2 += k[q] * conc[nc - w] + (1.0 - k[q]) * conc[nc];
                }
                /* (the reference stores (t - h*fac[srow_prev + w1]) / d here
                 * and overwrites it with t / d below) */
                part[pr] = (t2 + k[q] * part[pr - w] - h * part[prev_shell]) / d;
                q += m < last ? 2 : 1;
            } else {
                d += 1.0 + k[q];
                fac[row + 1] = -k[q] / d;
                part[pr] = (t2 + (1.0 - k[q]) * conc[nc] + k[q] * conc[nc + w]) / d;
                q++;
            }
            fac[row] = t / d;
            pr++;
            nc++;
            row += w;
        }
        /* the shell row */
        if (m) {
            if (m < last) {
                dsh += k[q + 1] + k[q] * (1.0 + fac[srow_prev + w1]);
                rsh += k[q] * (conc[nc - w] + part[prev_shell]) + (1.0 - k[q] - k[q + 1]) * co;
                cs += w;
                co = conc[cs];
                rsh += k[q + 1] * co;
            } else {
                dsh += k[q] * (1.0 + fac[srow_prev + w1]);
                rsh += k[q] * (conc[nc - w] + part[prev_shell]) + (1.0 - k[q]) * co;
            }
        } else {
            dsh += k[q];
            rsh += (1.0 - k[q]) * co;
            cs += w;
            co = conc[cs];
            rsh += k[q] * co;
        }
        /* eliminate the buffer terms of the shell row */
        for (n = 0, nb = srow_prev; n < nfix; n++) {
            nb += w;
            prev_shell++;
            dsh -= fac[row + n] * fac[nb];
            rsh -= fac[row + n] * part[prev_shell];
        }
        for (; n < w1; n++) {
            double e;
            nb += w;
            prev_shell++;
            e = m ? fac[row + n] + k[q] * fac[srow_prev + n] : fac[row + n];
            dsh -= e * fac[nb];
            rsh -= e * part[prev_shell];
            if (m < last) fac[row + n] *= -fac[nb + 1];
        }
        if (m < last) {
            for (n = nfix; n < w1; n++) fac[row + n] /= dsh;
            if (m) {
                fac[row + w1] = -k[q + 1] / dsh;
                q += 2;
            } else {
                fac[row + w1] = -k[q] / dsh;
                q++;
            }
            part[pr] = rsh / dsh;
            prev_shell = pr++;
            nc++;
            srow_prev = row;
            srow += sq;
            row += w;
        } else {
            co = conc[nc] = rsh / dsh;
            nc--;
            q++;
        }
    }
    /* back substitution, outermost shell first */
    for (m = last; m >= 0; m--) {
        if (m < last) {
            row -= w;
            co = part[--pr] - fac[row + w1] * conc[nc + w];
            for (n = nfix; n < w1; n++) co -= fac[row + n] * conc[nc + n + 1];
            conc[nc] = co;
            nc--;
            for (n = w1; n > nfix; n--) {
                row -= w;
                conc[nc] = part[--pr] - fac[row] * co - fac[row + 1] * conc[nc + w];
                nc--;
            }
        } else {
            for (n = w1; n > nfix; n--) {
                row -= w;
                conc[nc] = part[--pr] - fac[row] * co;
                nc--;
            }
        }
        for (; n > 0; n--) {
            row -= w;
            conc[nc] = part[--pr] - fac[row] * co;
            nc--;
        }
    }
    *cursor = q;
}

void orc_conc_solve(orc_solver *s)
{
    int i, cursor = 0;
    for (i = 0; i < s->ndiffs; i++) {
        if (s->nshrows[i] > 1)
            diff_buffered(s, s->dconc[i], s->nshells[i], s->nshrows[i], s->nshfix[i], s->fbufval[i], &cursor);
        else
            diff_shells(s, s->dconc[i], s->nshells[i], &cursor);
    }
}

/*
 * Hines elimination over funcs[] (hines_solve.c:140-296). resultval/diaval
 * are the running row accumulators; 'cur' is the row-pair cursor into
 * results[]. crank: vm = 2x - vm, otherwise vm = x.
 */
void orc_solve(orc_solver *s)
{
    const int *f = s->funcs;
    double *res = s->results, *ra = s->ravals;
    double *vmv = s->vm;
    int vrow = s->ncompts - 1;
    int fi = 0, ri = 0, cur;
    double temp = 0.0, rv, dv;
    int op;

    op = f[fi++];
    if (s->ncompts == 1) {
        const double x = res[0] / res[1];
        if (s->crank) vmv[0] = x + x - vmv[0];
        else vmv[0] = x;
        return;
    }
    cur = 2;
    rv = res[cur];
    dv = res[cur + 1];
    for (;;) {
        if (op == F_ELIM) {
            temp = ra[ri++] / res[f[fi] + 1];
            dv -= ra[ri++] * temp;
            rv -= res[f[fi++]] * temp;
        } else if (op == F_SET_DIAG) {
            res[cur++] = rv;
            res[cur++] = dv;
            rv = res[cur];
            dv = res[cur + 1];
        } else if (op == F_SKIP_DIAG) {
            res[cur++] = rv;
            res[cur] = dv;
            cur += 3;
            rv = res[cur];
            dv = res[cur + 1];
        } else if (op == F_FASTSIB) {
            ra[f[fi++]] -= ra[ri++] * temp;
        } else if (op == F_COPY) {
            ra[f[fi++]] = ra[ri++];
        } else if (op == F_SIB) {
            ra[f[fi + 1]] -= ra[f[fi]] * temp;
            fi += 2;
        } else {
            break;
        }
        op = f[fi++];
    }
    rv = rv / dv;
    if (s->crank) vmv[vrow] = rv + rv - vmv[vrow];
    else vmv[vrow] = rv;
    res[cur] = rv;
    cur -= 2;
    rv = res[cur];
    for (;;) {
        op = f[fi++];
        if (op == F_ELIM) {
            rv -= ra[ri++] * res[f[fi++]];
        } else if (op == F_CALC) {
            rv = rv / res[cur + 1];
            vrow--;
            if (s->crank) vmv[vrow] = rv + rv - vmv[vrow];
            else vmv[vrow] = rv;
            res[cur] = rv;
            cur -= 2;
            if (cur >= 0) rv = res[cur];   /* the reference reads one row below results[] here */
        } else if (op == F_SIB) {
            rv -= ra[f[fi]] * res[f[fi + 1]];
            fi += 2;
        } else {
            break;
        }
    }
}

int orc_process(orc_solver *s)
{
    if (orc_chip_update(s)) return -1;
    if (s->nconcchips_used) {
        if (orc_conc_update(s)) return -1;
    }
    if (s->ndiffs) orc_conc_solve(s);
    orc_solve(s);
    return 0;
}

int orc_run_loss(orc_solver *s, int nsteps, int ntargets, const int *rows, const double *trace, double *loss)
{
    int i, j;
    double sum = 0.0;
    for (i = 0; i < nsteps; i++) {
        if (orc_process(s)) return -1;
        for (j = 0; j < ntargets; j++) {
            const double d = s->vm[rows[j]] - trace[(long)i * ntargets + j];
            sum += d * d;
        }
    }
    *loss = sum;
    return 0;
}

/* Runs nsteps steps recording vm[rows[j]] after every step into
 * out[i * nrows + j], and the voltage-table row each compartment's Vm falls
 * in after every step into tab_rows[i * ncompts + c] (NULL: not recorded). */
int orc_run_trace(orc_solver *s, int nsteps, int nrows, const int *rows, double *out, int *tab_rows)
{
    int i, j, c;
    for (i = 0; i < nsteps; i++) {
        if (orc_process(s)) return -1;
        for (j = 0; j < nrows; j++) out[(long)i * nrows + j] = s->vm[rows[j]];
        if (tab_rows)
            for (c = 0; c < s->ncompts; c++) {
                double f = (s->vm[c] - s->xmin) * s->invdx;
                if (f < 0.0) f = 0.0;
                else if (f > s->xdivs) f = s->xdivs;
                tab_rows[(long)i * s->ncompts + c] = (int)f;
            }
    }
    return 0;
}

int orc_run(orc_solver *s, int nsteps)
{
    int i;
    for (i = 0; i < nsteps; i++)
        if (orc_process(s)) return -1;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Network layer: spikes -> per-synchan pending events.                     */
/*                                                                          */
/* The reference keeps a delta-encoded pending list per synchan and a       */
/* countdown in ops[] (synchan.c:160-350, hines_conn.c:44-108). Restated    */
/* with absolute step numbers: an event created while source solver 'a'     */
/* runs step s, with delay d steps, fires at step s+d in a target solver    */
/* processed after 'a' in the same step (or 'a' itself), and at s+d+1 in a  */
/* target processed before 'a' (its countdown for step s is already spent). */
/* Events due on the same step are summed newest-first, which is the order  */
/* the reference's insert-before-equal list yields.                         */
/* ------------------------------------------------------------------------ */

typedef struct orc_event {
    long long fire_step;
    double weight;
    struct orc_event *next;
} orc_event;

typedef struct {
    int solver, child, op;  /* synchan identity: op = ops index of SYN2/3 */
    orc_event *head;        /* sorted by fire_step, newest first on ties */
} orc_synchan;

struct orc_net {
    int nsolvers;
    orc_solver **sv;
    const int *syn_start, *tgt_solver, *tgt_child, *tgt_op, *delay;
    const double *weight;
    int nsyn, cap_syn;      /* synchan table and its capacity */
    orc_synchan *syn;
    int *syn_of_synapse;    /* synapse -> synchan table index */
    long long step;
    int cur_solver;
    int (*process)(orc_solver *);
    long long *spike_counts;
};

static int orc_find_synchan(orc_net *n, int solver, int child, int op)
{
    int i;
    for (i = 0; i < n->nsyn; i++)
        if (n->syn[i].solver == solver && n->syn[i].child == child) return i;
    if (n->nsyn == n->cap_syn) {
        n->cap_syn = 2 * n->cap_syn + 8;
        n->syn = (orc_synchan *)realloc(n->syn, (size_t)n->cap_syn * sizeof(orc_synchan));
    }
    n->syn[n->nsyn].solver = solver;
    n->syn[n->nsyn].child = child;
    n->syn[n->nsyn].op = op;
    n->syn[n->nsyn].head = NULL;
    return n->nsyn++;
}

static void orc_net_on_spike(void *ctx, int solver_id)
{
    orc_net *n = (orc_net *)ctx;
    int e;
    if (n->spike_counts) n->spike_counts[solver_id]++;
    for (e = n->syn_start[solver_id]; e < n->syn_start[solver_id + 1]; e++) {
        orc_synchan *sc = &n->syn[n->syn_of_synapse[e]];
        orc_solver *t = n->sv[sc->solver];
        long long fire = n->step + n->delay[e] + (sc->solver < solver_id ? 1 : 0);
        orc_event *ev = (orc_event *)malloc(sizeof(orc_event));
        orc_event **pp = &sc->head;
        ev->fire_step = fire;
        ev->weight = n->weight[e];
        while (*pp && (*pp)->fire_step < fire) pp = &(*pp)->next;
        ev->next = *pp;
        *pp = ev;
        if (sc->head == ev) {
            /* new first event: reset the countdown (HSEVENT, hines.c:352-357);
             * the countdown is consumed once per step by SYN2_OP */
            long long base = n->step + (sc->solver < solver_id ? 1 : 0);
            t->ops[sc->op + 2] = (int)(fire - base);
        }
    }
}

static int orc_net_on_syn(void *ctx, int solver_id, int stab, int child, int x_slot)
{
    orc_net *n = (orc_net *)ctx;
    orc_solver *s = n->sv[solver_id];
    int i;
    double activation = 0.0;
    orc_synchan *sc = NULL;
    for (i = 0; i < n->nsyn; i++)
        if (n->syn[i].solver == solver_id && n->syn[i].child == child) { sc = &n->syn[i]; break; }
    if (!sc) return -1;
    /* HPROCESS: fire every event due now, newest first (synchan.c:307-350) */
    while (sc->head && sc->head->fire_step <= n->step) {
        orc_event *ev = sc->head;
        sc->head = ev->next;
        activation += ev->weight / s->dt;
        free(ev);
    }
    /* h_dosynchan (hines_conn.c:62-89) */
    s->chip[x_slot] += s->dt * activation * s->stablist[stab + 3];
    if (sc->head) return (int)(sc->head->fire_step - n->step);
    return -1;
}

orc_net *orc_net_create(int nsolvers, orc_solver **solvers, const int *syn_start,
                        const int *syn_target_solver, const int *syn_target_child,
                        const int *syn_target_op, const double *syn_weight,
                        const int *syn_delay_steps)
{
    orc_net *n = (orc_net *)calloc(1, sizeof(orc_net));
    int nsynapses = syn_start[nsolvers], e, i;
    n->nsolvers = nsolvers;
    n->sv = solvers;
    n->syn_start = syn_start;
    n->tgt_solver = syn_target_solver;
    n->tgt_child = syn_target_child;
    n->tgt_op = syn_target_op;
    n->weight = syn_weight;
    n->delay = syn_delay_steps;
    n->process = orc_process;
    n->cap_syn = nsynapses + 1;
    n->syn = (orc_synchan *)calloc(n->cap_syn, sizeof(orc_synchan));
    n->syn_of_synapse = (int *)calloc(nsynapses + 1, sizeof(int));
    for (e = 0; e < nsynapses; e++)
        n->syn_of_synapse[e] = orc_find_synchan(n, syn_target_solver[e], syn_target_child[e],
                                                syn_target_op[e]);
    for (i = 0; i < nsolvers; i++) {
        solvers[i]->id = i;
        solvers[i]->on_spike = orc_net_on_spike;
        solvers[i]->on_syn = orc_net_on_syn;
        solvers[i]->hook_ctx = n;
    }
    return n;
}

void orc_net_destroy(orc_net *n)
{
    int i;
    if (!n) return;
    for (i = 0; i < n->nsyn; i++) {
        orc_event *ev = n->syn[i].head;
        while (ev) { orc_event *nx = ev->next; free(ev); ev = nx; }
    }
    free(n->syn);
    free(n->syn_of_synapse);
    free(n);
}

int orc_net_run(orc_net *n, int nsteps, long long *spike_counts)
{
    int t, i;
    n->spike_counts = spike_counts;
    for (t = 0; t < nsteps; t++) {
        for (i = 0; i < n->nsolvers; i++) {
            n->cur_solver = i;
            if (n->process(n->sv[i])) return -1;
        }
        n->step++;
    }
    return 0;
}

long long orc_net_step_count(const orc_net *n) { return n->step; }

/* Events from spikes outside the network (other ranks of a partitioned run),
 * added after a step: event k acts on the synchan (tgt_solver, tgt_child,
 * op tgt_op) in step fire_step (> the step just run), with weight w. Queue
 * order and countdown as orc_net_on_spike, counted from the next step. */
void orc_net_deliver(orc_net *n, int count, const int *tgt_solver, const int *tgt_child, const int *tgt_op,
                     const double *w, const long long *fire_step)
{
    int k;
    for (k = 0; k < count; k++) {
        orc_synchan *sc = &n->syn[orc_find_synchan(n, tgt_solver[k], tgt_child[k], tgt_op[k])];
        orc_solver *t = n->sv[sc->solver];
        orc_event *ev = (orc_event *)malloc(sizeof(orc_event));
        orc_event **pp = &sc->head;
        ev->fire_step = fire_step[k];
        ev->weight = w[k];
        while (*pp && (*pp)->fire_step < fire_step[k]) pp = &(*pp)->next;
        ev->next = *pp;
        *pp = ev;
        if (sc->head == ev) t->ops[sc->op + 2] = (int)(fire_step[k] - n->step);
    }
}

void orc_net_set_process(orc_net *n, int (*process)(orc_solver *)) { n->process = process; }
