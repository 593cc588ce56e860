/*
 * adapter_host.c -- a minimal GENESIS host for the engine's GENESIS adapter
 * (genesis-2.4_gb300/adapter/gbh_hsolve_adapter.c). TEST INFRASTRUCTURE.
 *
 * Compiled together with the adapter against the reference's own headers
 * (hines_ext.h and what it includes), it supplies the parts of GENESIS the
 * adapter touches:
 *   simulation_time   -- the simulation clock (sim/sim_ext.h:38), read by
 *                        SimulationTime() for the step stamp
 *   BaseObject()      -- the element's object, whose method field names the
 *                        integration method (11 = Crank-Nicolson)
 *   IsHsolved(), CallEventAction()
 *                     -- spike targets; this host builds no spikegen, so
 *                        neither is reached
 *   h_in_msgs messages -- one Msg followed by its Slot, whose func returns the
 *                        message's value (MSGVALUE, sim/sim_defs.h:264,274)
 * It builds an Hsolve around the arrays of the oracle's solver struct and
 * runs PROCESS as hines.c does with the accelerator bound
 * (hines.c:253-268): gbh_chip_update, which returns 1 when the step is done
 * (conc update and solve included).
 */
#include <stdlib.h>
#include <string.h>

#include "hines_ext.h"
#include "gbh_hsolve.h"
#include "hsolve_oracle.h"

extern int gbh_init(Hsolve *h);
extern int gbh_chip_update(Hsolve *h);
extern void gbh_sync_chip(Hsolve *h);
extern int gbh_push_state(Hsolve *h);
extern void gbh_cleanup(void);

double simulation_time;

static GenesisObject host_euler, host_crank;

GenesisObject *BaseObject(Element *e) { return e->object; }
int IsHsolved(Element *e) { (void)e; return 0; }
int CallEventAction(void) { return 0; }

/* an incoming message with one slot holding a double */
typedef struct host_msg {
    Msg m;
    Slot slot[1];
} host_msg;

static double host_slot_value(Slot *s) { return *(double *)s->data; }

typedef struct host_solver {
    Hsolve h;
    Oinfo out;
    int *fcoval;
    Iinfo *in;
    host_msg *msg;
} host_solver;

/* An Hsolve over the oracle struct's arrays (borrowed), with ninject INJECT
 * messages onto chip rows rows[k] whose values are read from values[k] at
 * every step, and output messages when has_outputs is set. */
void *ah_create(orc_solver *s, const char *name, int nstab_doubles, int ncovals0, int ninject, const int *rows,
                double *values, int has_outputs)
{
    host_solver *hs = (host_solver *)calloc(1, sizeof(host_solver));
    Hsolve *h = &hs->h;
    int k;
    host_euler.method = 0;
    host_crank.method = CRANK_INT;
    h->name = (char *)name;
    h->object = s->crank ? &host_crank : &host_euler;
    h->dt = s->dt;
    h->chanmode = s->chanmode;
    h->calcmode = s->calcmode;
    h->storemode = s->storemode;
    h->ncompts = s->ncompts;
    h->nops = s->nops;         h->ops = s->ops;
    h->nchips = s->nchips;     h->chip = s->chip;
    h->nfuncs = s->nfuncs;     h->funcs = s->funcs;
    h->nravals = s->nravals;   h->ravals = s->ravals;
    h->vm = s->vm;
    h->ngivals = s->ngivals;   h->givals = s->givals;
    h->sntab = nstab_doubles / SYNSIZE;
    h->stablist = s->stablist;
    h->nconcs = s->nconcs;     h->conc = s->conc;
    h->nconcchips = s->nconcchips_used ? s->nconcchips : 0;
    h->nconcops = s->nconcops; h->concops = s->concops;
    h->concchip = s->concchip;
    h->ncols = s->ncols;       h->xdivs = s->xdivs;   h->ydivs = s->ydivs;
    h->xmin = s->xmin;         h->invdx = s->invdx;
    h->ymin = s->ymin;         h->invdy = s->invdy;
    h->tablist = s->tablist;   h->xvals = s->xvals;   h->yvals = s->yvals;
    h->childops = s->childops; h->childchips = s->childchips;
    if (s->ndiffs) {
        /* only fcoval[ndiffs], the length of covals0, is read */
        hs->fcoval = (int *)calloc(s->ndiffs + 1, sizeof(int));
        hs->fcoval[s->ndiffs] = ncovals0;
        h->ndiffs = s->ndiffs;
        h->dconc = s->dconc;   h->nshells = s->nshells;   h->nshrows = s->nshrows;
        h->nshfix = s->nshfix; h->fbufval = s->fbufval;   h->fcoval = hs->fcoval;
        h->covals0 = s->covals0;
        h->bufvals = s->bufvals;
    }
    if (s->storemode) {
        h->itotal = s->itotal;
        h->nelm_names = s->nelm_names;
    }
    if (has_outputs) h->outinfo = &hs->out;
    if (ninject > 0) {
        hs->in = (Iinfo *)calloc(ninject, sizeof(Iinfo));
        hs->msg = (host_msg *)calloc(ninject, sizeof(host_msg));
        for (k = 0; k < ninject; k++) {
            hs->msg[k].m.nslots = 1;
            hs->msg[k].slot[0].data = (char *)&values[k];
            hs->msg[k].slot[0].func = (PFD)host_slot_value;
            hs->in[k].type = INJECT_OP;
            hs->in[k].msgin = &hs->msg[k].m;
            hs->in[k].nchip = rows[k];
            hs->in[k].next = k + 1 < ninject ? &hs->in[k + 1] : NULL;
        }
        h->ininfo = &hs->in[0];
    }
    return hs;
}

int ah_init(void *p) { return gbh_init(&((host_solver *)p)->h); }

/* PROCESS of one solver at simulation time t */
int ah_process(void *p, double t)
{
    simulation_time = t;
    return gbh_chip_update(&((host_solver *)p)->h);
}

void ah_sync(void *p) { gbh_sync_chip(&((host_solver *)p)->h); }

int ah_push(void *p) { return gbh_push_state(&((host_solver *)p)->h); }

/* gbh_cleanup, then the host's own allocations */
void ah_destroy_all(void **p, int n)
{
    int k;
    gbh_cleanup();
    for (k = 0; k < n; k++) {
        host_solver *hs = (host_solver *)p[k];
        free(hs->fcoval);
        free(hs->in);
        free(hs->msg);
        free(hs);
    }
}
