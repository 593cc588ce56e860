/*
 * ref_shim.c -- binds the reference's own chanmode 4/5 step functions to the
 * oracle's flat-array solver struct.
 *
 * TEST INFRASTRUCTURE ONLY. Compiled together with the reference sources
 * genesis/src/hines/{hines_4chip,hines_4nichip,hines_conc_4chip,hines_conc,hines_solve}.c
 * (never copied into this repository) into oracle/_ref/libhsolve_ref.so by
 * oracle/Makefile, and used to pin the oracle restatement bit for bit.
 *
 * It supplies the symbols those files need from the rest of GENESIS:
 *   Error()            -- message banner (sim/)
 *   the option-parsing symbols of sim/sim_random.c, whose G_RNG (the
 *                         uniform deviate SYN3_OP draws) is linked in as is
 *   h_dospike_event()  -- hines_conn.c:44-58, routed to the solver's hook
 *   h_dosynchan()      -- hines_conn.c:62-89, routed to the solver's hook
 *   BaseObject()       -- the element's object, for its integration method
 * and builds a transient Hsolve around the oracle struct's arrays for each call.
 */
#include <stdlib.h>
#include <string.h>
#include "hines_ext.h"
#include "hsolve_oracle.h"

extern int do_chip_hh4_update(Hsolve *);
extern int do_chip_hh4ni_update(Hsolve *);
extern int do_h4_conc_chip_update(Hsolve *);
extern void do_euler_hsolve(Hsolve *);
extern void do_crank_hsolve(Hsolve *);
extern void do_h_conc_solve(Hsolve *);

void Error(void) {}

/* do_h_conc_solve reads the integration method from the element's object
 * (sim/sim_func_ext.h:258); one static object carries the current solver's */
static GenesisObject ref_object;
GenesisObject *BaseObject(Element *e)
{
    (void)e;
    return &ref_object;
}

/* G_RNG / G_SEEDRNG come from the reference's own sim/sim_random.c, linked
 * beside this file; its option parsing (do_setRNG) is never called here and
 * needs only these symbols */
char *G_optopt;
int G_getopt() { return -1; }
int initopt() { return 0; }
void printoptusage() {}
int IsSilent() { return 1; }

void h_dospike_event(Hsolve *hsolve)
{
    orc_solver *s = (orc_solver *)hsolve->accel_state;
    if (s && s->on_spike) s->on_spike(s->hook_ctx, s->id);
}

void h_dosynchan(Hsolve *hsolve, int stabindex, int cindex)
{
    orc_solver *s = (orc_solver *)hsolve->accel_state;
    int nop = hsolve->childops[cindex];
    int nchip = hsolve->childchips[cindex];
    if (hsolve->ops[nop] == SYN3_OP) nchip++;
    if (s && s->on_syn)
        hsolve->ops[nop + 2] = s->on_syn(s->hook_ctx, s->id, stabindex, cindex, nchip);
    else
        hsolve->ops[nop + 2] = -1;
}

static void ref_fill(Hsolve *h, orc_solver *s)
{
    memset(h, 0, sizeof(*h));
    h->ncompts = s->ncompts;
    h->chanmode = s->chanmode;
    h->calcmode = s->calcmode;
    h->storemode = s->storemode;
    h->ops = s->ops;
    h->nops = s->nops;
    h->chip = s->chip;
    h->nchips = s->nchips;
    h->funcs = s->funcs;
    h->nfuncs = s->nfuncs;
    h->ravals = s->ravals;
    h->nravals = s->nravals;
    h->results = s->results;
    h->vm = s->vm;
    h->vmlast = s->vm + s->ncompts - 1;
    h->givals = s->givals;
    h->ngivals = s->ngivals;
    h->ovals = s->ovals;
    h->tablist = s->tablist;
    h->ncols = s->ncols;
    h->xdivs = s->xdivs;
    h->xmin = s->xmin;
    h->invdx = s->invdx;
    h->xvals = s->xvals;
    h->ydivs = s->ydivs;
    h->ymin = s->ymin;
    h->invdy = s->invdy;
    h->yvals = s->yvals;
    h->stablist = s->stablist;
    h->nconcs = s->nconcs;
    h->conc = s->conc;
    h->flux = s->flux;
    h->codiag = s->codiag;
    h->coresult = s->coresult;
    h->nconcchips = s->nconcchips_used ? s->nconcchips : 0;
    h->concchip = s->concchip;
    h->nconcops = s->nconcops;
    h->concops = s->concops;
    h->itotal = s->itotal;
    h->nelm_names = s->nelm_names;
    h->ndiffs = s->ndiffs;
    h->dconc = s->dconc;
    h->nshells = s->nshells;
    h->nshrows = s->nshrows;
    h->nshfix = s->nshfix;
    h->fbufval = s->fbufval;
    h->covals0 = s->covals0;
    h->bufvals = s->bufvals;
    h->covals = s->covals;
    h->cores = s->cores;
    h->childops = s->childops;
    h->childchips = s->childchips;
    h->dt = s->dt;
    h->accel_state = s;
}

/* One PROCESS step, chanmode 4/5 CPU branch of hines.c:253-268. */
int ref_process(orc_solver *s)
{
    Hsolve h;
    int rc;
    ref_fill(&h, s);
    rc = s->calcmode ? do_chip_hh4_update(&h) : do_chip_hh4ni_update(&h);
    if (rc) return -1;
    if (h.nconcchips) {
        if (do_h4_conc_chip_update(&h)) return -1;
    }
    if (h.ndiffs) {
        ref_object.method = s->crank ? CRANK_INT : BEULER_INT;
        do_h_conc_solve(&h);
    }
    if (s->crank)
        do_crank_hsolve(&h);
    else
        do_euler_hsolve(&h);
    return 0;
}

int ref_run(orc_solver *s, int nsteps)
{
    int i;
    for (i = 0; i < nsteps; i++)
        if (ref_process(s)) return -1;
    return 0;
}
