/*
 * gbh_hsolve_adapter.c -- the GENESIS side of the GB300 engine.
 *
 * Compiled INSIDE a GENESIS build (it includes the reference's hines_ext.h)
 * in place of genesis/src/hines/cuda/cuda_hsolve.c. It exposes the same four
 * entry points the reference's accelerator macro binds
 * (genesis/src/hines/cuda/cuda_hsolve.h:22-25, selected in
 * genesis/src/hines/hines.c:93-98):
 *
 *   int  gbh_init(Hsolve *)          -- cuda_init:        registers the solver
 *   int  gbh_chip_update(Hsolve *)   -- cuda_chip_update: one whole PROCESS
 *                                       step on the GPU; returns 1 (vm ready)
 *   void gbh_sync_chip(Hsolve *)     -- cuda_sync_chip:   device -> chip/vm/conc
 *   void gbh_cleanup(void)           -- cuda_cleanup
 *
 * plus one the reference has no counterpart for:
 *
 *   int  gbh_push_state(Hsolve *)    -- chip/vm/conc -> device, after the host
 *                                       wrote them (RESTORE2, hines.c:560-571;
 *                                       HPUT; RESET's element values)
 *
 * Every solver joins one batch engine through the GENESIS-free hsolve-level
 * ABI (include/gbh_hsolve.h): the first gbh_chip_update call of a simulation
 * step runs every registered solver, later calls in that step return at once
 * (the reference batches the same way, cuda_hsolve.c:64-145, but only
 * without spike detectors). The engine runs the chip update, the Ca pools
 * and the Hines elimination, so hines.c must skip do_h4_conc_chip_update and
 * the CPU solve when gbh_chip_update returns 1.
 *
 * Inputs: the h_in_msgs targets listed in hsolve->ininfo (INJECT, BASE,
 * THRESH, SYN2, FLUX) are read from their messages at each step and applied
 * on the device. Outputs: a solver with output messages (hsolve->outinfo)
 * gets its vm (and itotal) back after every step, for h_out_msgs. Spikes: a
 * solver's spikegen messages to synchans of solvers in the batch become
 * device synapses (weight and delay from the synapse entry, synchan.c:
 * 160-240); messages to any other element are sent on the host
 * (CallEventAction, as h_dospike_event does) for every spike.
 */
#include <stdlib.h>
#include <string.h>

#include "hines_ext.h"
#include "gbh_hsolve.h"

#define GBH_MAX_SOLVERS (1 << 20)

typedef struct gbh_hstate {
    int id;                     /* hsolve-level id */
    gbh_hs_input *in;
    int nin;
    gbh_hs_synapse *syn;        /* resolved before the first step */
    int nsyn;
    int resolved;
} gbh_hstate;

static Hsolve **gbh_registry = NULL;
static int gbh_nreg = 0, gbh_cap = 0;
static int gbh_synapses_resolved = 0;

/* value of an h_in_msgs message (hines_msgs.c:351-405) */
static double gbh_msg_value(void *ctx)
{
    Iinfo *ii = (Iinfo *)ctx;
    return MSGVALUE(ii->msgin, 0);
}

static int gbh_in_batch(Element *dst, int *id_out, int *op_out, int *syn_out, MsgOut *mo)
{
    S2chan *ch;
    Hsolve *th;
    gbh_hstate *ts;
    int i;
    if (!dst || !IsHsolved(dst)) return 0;
    ch = (S2chan *)dst;
    th = (Hsolve *)ch->hsolve;
    if (!th || !th->accel_state) return 0;
    ts = (gbh_hstate *)th->accel_state;
    for (i = 0; i < ch->nsynapses; i++)
        if (ch->synapse[i].mi == (MsgIn *)mo) break;
    if (i == ch->nsynapses) return 0;
    *id_out = ts->id;
    *op_out = th->childops[ch->solve_index];
    *syn_out = i;
    return 1;
}

/* spikegen messages to elements outside the batch, on the host */
static void gbh_host_spike(void *ctx)
{
    Hsolve *h = (Hsolve *)ctx;
    struct Spikegen_type *spike = (struct Spikegen_type *)h->spikegen;
    MsgOut *mo;
    int id, op, si;
    MSGOUTLOOP(spike, mo) {
        if (!gbh_in_batch(mo->dst, &id, &op, &si, mo)) CallEventAction(spike, mo);
    }
    spike->lastevent = SimulationTime();
}

/* Synapses of every solver's spikegen onto synchans of the batch: their
 * targets are registered by the time the first step runs. */
static int gbh_resolve_synapses(void)
{
    int k;
    for (k = 0; k < gbh_nreg; k++) {
        Hsolve *h = gbh_registry[k];
        gbh_hstate *s = (gbh_hstate *)h->accel_state;
        struct Spikegen_type *spike;
        MsgOut *mo;
        int n = 0, host = 0, id, op, si;
        if (!s || !h->spikegen) continue;
        spike = (struct Spikegen_type *)h->spikegen;
        MSGOUTLOOP(spike, mo) {
            if (gbh_in_batch(mo->dst, &id, &op, &si, mo)) n++;
            else host = 1;
        }
        free(s->syn);
        s->syn = (gbh_hs_synapse *)calloc(n ? n : 1, sizeof(gbh_hs_synapse));
        s->nsyn = 0;
        MSGOUTLOOP(spike, mo) {
            if (gbh_in_batch(mo->dst, &id, &op, &si, mo)) {
                S2chan *ch = (S2chan *)mo->dst;
                gbh_hs_synapse *y = &s->syn[s->nsyn++];
                y->target = id;
                y->target_op = op;
                y->weight = ch->synapse[si].weight;
                /* steps until the spike hits (synchan.c:199-200) */
                y->delay_steps = (int)(ch->synapse[si].delay / h->dt + 0.9);
            }
        }
        if (gbh_hs_set_synapses(s->id, s->nsyn, s->syn, host ? gbh_host_spike : NULL, h) != GBH_OK) return -1;
    }
    gbh_synapses_resolved = 1;
    return 0;
}

int gbh_init(Hsolve *h)
{
    gbh_hs_solver d;
    gbh_hstate *s;
    Iinfo *ii;
    int n, i;

    if (h->accel_state) return 0;
    memset(&d, 0, sizeof(d));
    d.dt = h->dt;
    d.method = BaseObject(h)->method;   /* 11 = CRANK_INT, else backward Euler */
    d.chanmode = h->chanmode;
    d.calcmode = h->calcmode;
    d.storemode = h->storemode;
    d.ncompts = h->ncompts;
    d.nops = h->nops;        d.ops = h->ops;
    d.nchips = h->nchips;    d.chip = h->chip;
    d.nfuncs = h->nfuncs;    d.funcs = h->funcs;
    d.nravals = h->nravals;  d.ravals = h->ravals;
    d.vm = h->vm;
    d.ngivals = h->ngivals;  d.givals = h->givals;
    d.nstab = h->sntab * SYNSIZE;
    d.stablist = h->stablist;
    d.nconcs = h->nconcs;    d.conc = h->conc;
    d.nconcops = h->nconcchips ? h->nconcops : 0;
    d.concops = h->concops;
    d.nconcchips = h->nconcchips;
    d.concchip = h->concchip;
    d.tables.ncols = h->ncols;
    d.tables.xdivs = h->xdivs;
    d.tables.ydivs = h->ydivs;
    d.tables.xmin = h->xmin;
    d.tables.invdx = h->invdx;
    d.tables.ymin = h->ymin;
    d.tables.invdy = h->invdy;
    d.tables.tablist = h->tablist;
    d.tables.xvals = h->xvals;
    d.tables.yvals = h->yvals;
    if (h->ndiffs) {   /* difshell systems (h_init_conc_solve / h_setup_conc_solve) */
        d.ndiffs = h->ndiffs;
        d.dconc = h->dconc;
        d.nshells = h->nshells;
        d.nshrows = h->nshrows;
        d.nshfix = h->nshfix;
        d.fbufval = h->fbufval;
        d.ncovals0 = h->fcoval[h->ndiffs];
        d.covals0 = h->covals0;
        d.nbufvals = h->fbufval[h->ndiffs];
        d.bufvals = h->bufvals;
    }
    if (h->storemode && h->itotal) {   /* itotal[nelm_names] (hines_chip_init.c:753) */
        d.nelm_names = h->nelm_names;
        d.itotal = h->itotal;
    }
    d.has_outputs = h->outinfo != NULL;
    s = (gbh_hstate *)calloc(1, sizeof(*s));
    /* h_in_msgs inputs (hines_msgs.c:351-405): INJECT/BASE/THRESH set a chip,
       SYN2 adds to a synchan's X, FLUX sets a concentration's flux */
    n = 0;
    for (ii = h->ininfo; ii; ii = ii->next)
        if (ii->type == INJECT_OP || ii->type == BASE_OP || ii->type == THRESH_OP || ii->type == SYN2_OP ||
            ii->type == FLUX_OP)
            n++;
    s->in = (gbh_hs_input *)calloc(n ? n : 1, sizeof(gbh_hs_input));
    i = 0;
    for (ii = h->ininfo; ii; ii = ii->next) {
        gbh_hs_input *in = &s->in[i];
        if (ii->type == INJECT_OP || ii->type == BASE_OP || ii->type == THRESH_OP) {
            in->kind = GBH_IN_SET;
            in->sa = in->sb = 1.0;
        } else if (ii->type == SYN2_OP) {
            in->kind = GBH_IN_ADD;
            in->sa = h->stablist[ii->nop + 3];
            in->sb = (ii->msgin->type == ACTIVATION && ii->sChildType == SYNCHANC_T) ? h->dt : 1.0;
        } else if (ii->type == FLUX_OP) {
            in->kind = GBH_IN_FLUX;
            in->sa = in->sb = 1.0;
        } else {
            continue;
        }
        in->index = ii->nchip;
        in->value = gbh_msg_value;
        in->ctx = ii;
        i++;
    }
    s->nin = i;
    d.ninputs = s->nin;
    d.inputs = s->in;
    s->id = gbh_hs_register(&d);
    if (s->id < 0) {
        fprintf(stderr, "gbh_init %s: could not register the solver\n", h->name);
        free(s->in);
        free(s);
        return -1;   /* hard SETUP error: there is no CPU fallback */
    }
    h->accel_state = s;
    if (gbh_nreg == gbh_cap) {
        gbh_cap = gbh_cap ? 2 * gbh_cap : 1024;
        if (gbh_cap > GBH_MAX_SOLVERS) return -1;
        gbh_registry = (Hsolve **)realloc(gbh_registry, gbh_cap * sizeof(Hsolve *));
    }
    gbh_registry[gbh_nreg++] = h;
    gbh_synapses_resolved = 0;
    return 0;
}

int gbh_chip_update(Hsolve *h)
{
    gbh_hstate *s;
    int rc;
    if (!h->accel_state && gbh_init(h)) return -1;
    if (!gbh_synapses_resolved && gbh_resolve_synapses()) return -1;
    s = (gbh_hstate *)h->accel_state;
    /* every solver of the batch gets the same stamp within a step */
    rc = gbh_hs_step(s->id, (long long)(SimulationTime() / h->dt + 0.5));
    if (rc < 0) {
        fprintf(stderr, "gbh_chip_update %s: %s\n", h->name, gbh_last_error());
        return -1;
    }
    return 1;   /* vm is ready: hines.c skips the conc update and the CPU solve */
}

void gbh_sync_chip(Hsolve *h)
{
    gbh_hstate *s = (gbh_hstate *)h->accel_state;
    if (s) gbh_hs_sync(s->id);
}

int gbh_push_state(Hsolve *h)
{
    gbh_hstate *s = (gbh_hstate *)h->accel_state;
    if (!s) return 0;   /* not registered yet: the batch copies the host arrays */
    if (gbh_hs_push(s->id) != GBH_OK) {
        fprintf(stderr, "gbh_push_state %s: %s\n", h->name, gbh_last_error());
        return -1;
    }
    return 0;
}

void gbh_cleanup(void)
{
    int k;
    gbh_hs_cleanup();
    for (k = 0; k < gbh_nreg; k++) {
        Hsolve *h = gbh_registry[k];
        gbh_hstate *s = (gbh_hstate *)h->accel_state;
        if (!s) continue;
        free(s->in);
        free(s->syn);
        free(s);
        h->accel_state = NULL;
    }
    free(gbh_registry);
    gbh_registry = NULL;
    gbh_nreg = gbh_cap = 0;
    gbh_synapses_resolved = 0;
}
