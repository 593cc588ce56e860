/*
 * gbh_hsolve_adapter.c -- the GENESIS side of the GB300 engine.
 *
 * Compiled INSIDE a GENESIS build (it includes the reference's hines_ext.h)
 * in place of genesis/src/hines/cuda/cuda_hsolve.c. It exposes the same four
 * entry points the reference's accelerator macro binds
 * (genesis/src/hines/cuda/cuda_hsolve.h:22-25, selected in
 * genesis/src/hines/hines.c:93-98):
 *
 *   int  gbh_init(Hsolve *)          -- cuda_init:        builds the engine
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
 * and maps one Hsolve onto the array-level C ABI of include/gbhsolve.h. The
 * engine runs the chip update, the Ca pools and the Hines elimination, so
 * hines.c must skip do_h4_conc_chip_update and the CPU solve when
 * gbh_chip_update returns 1.
 *
 * Per step it forwards the values h_in_msgs wrote into chip[] (INJECT, BASE,
 * THRESH targets listed in hsolve->ininfo) and, when the solver has output
 * messages (hsolve->outinfo), copies vm[] back so h_out_msgs sees current
 * values. Solvers holding spikegens or synchans that exchange events through
 * GENESIS messages must be batched through gbh_batch_desc + gbh_synapses by
 * the caller instead; gbh_init refuses them.
 */
#include <stdlib.h>
#include <string.h>

#include "hines_ext.h"
#include "gbhsolve.h"

#define GBH_MAX_SOLVERS 65536

typedef struct gbh_hstate {
    gbh_engine *e;
    int nin;
    Iinfo **in_msg;      /* the ininfo entry of every registered input */
    double *in_vals;
    int64_t starts[14][2];
} gbh_hstate;

static Hsolve *gbh_registry[GBH_MAX_SOLVERS];
static int gbh_nreg = 0;

static int gbh_fill_desc(Hsolve *h, gbh_batch_desc *d, gbh_tables *t, int *scalars /* [5] */,
                         int64_t (*st)[2])
{
    memset(d, 0, sizeof(*d));
    memset(t, 0, sizeof(*t));
    t->ncols = h->ncols;
    t->xdivs = h->xdivs;
    t->ydivs = h->ydivs;
    t->xmin = h->xmin;
    t->invdx = h->invdx;
    t->ymin = h->ymin;
    t->invdy = h->invdy;
    t->tablist = h->tablist;
    t->xvals = h->xvals;
    t->yvals = h->yvals;
    scalars[0] = BaseObject(h)->method;   /* 11 = CRANK_INT, else backward Euler */
    scalars[1] = h->chanmode;
    scalars[2] = h->calcmode;
    scalars[3] = 0;
    scalars[4] = h->storemode;
    d->abi_version = GBH_ABI_VERSION;
    d->nsolvers = 1;
    d->dt = h->dt;
    d->method = &scalars[0];
    d->chanmode = &scalars[1];
    d->calcmode = &scalars[2];
    d->table_set = &scalars[3];
    d->ntables = 1;
    d->tables = t;
#define GBH_RANGE(k, field, n) st[k][0] = 0; st[k][1] = (n); d->field##_start = st[k]; d->field = h->field
    GBH_RANGE(0, ops, h->nops);
    GBH_RANGE(1, chip, h->nchips);
    GBH_RANGE(2, funcs, h->nfuncs);
    GBH_RANGE(3, ravals, h->nravals);
    GBH_RANGE(4, vm, h->ncompts);
    GBH_RANGE(5, givals, h->ngivals);
    GBH_RANGE(7, conc, h->nconcs);
    GBH_RANGE(8, concops, h->nconcchips ? h->nconcops : 0);
    GBH_RANGE(9, concchip, h->nconcchips);
#undef GBH_RANGE
    st[6][0] = 0;
    st[6][1] = (int64_t)h->sntab * SYNSIZE;
    d->stab_start = st[6];
    d->stablist = h->stablist;
    if (h->ndiffs) {   /* difshell systems (h_init_conc_solve / h_setup_conc_solve) */
        st[10][0] = 0;
        st[10][1] = h->ndiffs;
        d->diff_start = st[10];
        d->dconc = h->dconc;
        d->nshells = h->nshells;
        d->nshrows = h->nshrows;
        d->nshfix = h->nshfix;
        d->fbufval = h->fbufval;
        st[11][0] = 0;
        st[11][1] = h->fcoval[h->ndiffs];
        d->covals0_start = st[11];
        d->covals0 = h->covals0;
        st[12][0] = 0;
        st[12][1] = h->fbufval[h->ndiffs];
        d->bufvals_start = st[12];
        d->bufvals = h->bufvals;
    }
    if (h->storemode && h->itotal) {   /* itotal[nelm_names] (hines_chip_init.c:753) */
        st[13][0] = 0;
        st[13][1] = h->nelm_names;
        d->storemode = &scalars[4];
        d->itotal_start = st[13];
    }
    return 0;
}

int gbh_init(Hsolve *h)
{
    gbh_batch_desc d;
    gbh_tables t;
    gbh_options opt;
    gbh_error err;
    int scalars[5];
    gbh_hstate *s;
    Iinfo *ii;
    int n, i;
    int *solver;
    int64_t *idx;

    if (h->accel_state) return 0;
    if (h->spikegen) {
        fprintf(stderr, "gbh_init %s: spike events need the batch API\n", h->name);
        return -1;
    }
    s = (gbh_hstate *)calloc(1, sizeof(*s));
    gbh_fill_desc(h, &d, &t, scalars, s->starts);
    memset(&opt, 0, sizeof(opt));
    s->e = gbh_create(&d, NULL, &opt, &err);
    if (!s->e) {
        fprintf(stderr, "gbh_init %s: solver %d row %d opcode %d: %s\n", h->name, err.solver, err.row, err.opcode,
                err.message);
        free(s);
        return -1;   /* hard SETUP error: there is no CPU fallback */
    }
    /* h_in_msgs inputs (hines_msgs.c:351-405): INJECT/BASE/THRESH set a chip,
       SYN2 adds to a synchan's X, FLUX sets a concentration's flux. The engine
       applies them itself from the message values, in ininfo order. */
    n = 0;
    for (ii = h->ininfo; ii; ii = ii->next)
        if (ii->type == INJECT_OP || ii->type == BASE_OP || ii->type == THRESH_OP || ii->type == SYN2_OP ||
            ii->type == FLUX_OP)
            n++;
    if (n) {
        int *kind = (int *)calloc(n, sizeof(int));
        double *sa = (double *)calloc(n, sizeof(double));
        double *sb = (double *)calloc(n, sizeof(double));
        s->nin = n;
        s->in_msg = (Iinfo **)calloc(n, sizeof(Iinfo *));
        s->in_vals = (double *)calloc(n, sizeof(double));
        solver = (int *)calloc(n, sizeof(int));
        idx = (int64_t *)calloc(n, sizeof(int64_t));
        i = 0;
        for (ii = h->ininfo; ii; ii = ii->next) {
            if (ii->type == INJECT_OP || ii->type == BASE_OP || ii->type == THRESH_OP) {
                kind[i] = GBH_IN_SET;
                sa[i] = sb[i] = 1.0;
            } else if (ii->type == SYN2_OP) {
                kind[i] = GBH_IN_ADD;
                sa[i] = h->stablist[ii->nop + 3];
                sb[i] = (ii->msgin->type == ACTIVATION && ii->sChildType == SYNCHANC_T) ? h->dt : 1.0;
            } else if (ii->type == FLUX_OP) {
                kind[i] = GBH_IN_FLUX;
                sa[i] = sb[i] = 1.0;
            } else {
                continue;
            }
            s->in_msg[i] = ii;
            idx[i] = ii->nchip;
            i++;
        }
        if (gbh_register_inputs_typed(s->e, n, solver, kind, idx, sa, sb) != GBH_OK)
            fprintf(stderr, "gbh_init %s: %s\n", h->name, gbh_last_error());
        free(solver);
        free(idx);
        free(kind);
        free(sa);
        free(sb);
    }
    h->accel_state = s;
    if (gbh_nreg < GBH_MAX_SOLVERS) gbh_registry[gbh_nreg++] = h;
    return 0;
}

int gbh_chip_update(Hsolve *h)
{
    gbh_hstate *s;
    int i;
    if (!h->accel_state && gbh_init(h)) return -1;
    s = (gbh_hstate *)h->accel_state;
    if (s->nin) {
        for (i = 0; i < s->nin; i++) s->in_vals[i] = MSGVALUE(s->in_msg[i]->msgin, 0);
        if (gbh_set_inputs_async(s->e, s->in_vals, NULL) != GBH_OK) return -1;
    }
    if (gbh_run(s->e, 1) != GBH_OK) {
        fprintf(stderr, "gbh_chip_update %s: %s\n", h->name, gbh_last_error());
        return -1;
    }
    if (h->outinfo && gbh_get_state(s->e, h->vm, NULL, NULL, NULL) != GBH_OK) return -1;
    if (h->outinfo && h->storemode && h->itotal && gbh_get_itotal(s->e, h->itotal) != GBH_OK) return -1;
    return 1;   /* vm is ready: hines.c skips the conc update and the CPU solve */
}

void gbh_sync_chip(Hsolve *h)
{
    gbh_hstate *s = (gbh_hstate *)h->accel_state;
    if (s) gbh_get_state(s->e, h->vm, h->chip, h->conc, h->ops);
    if (s && h->storemode && h->itotal) gbh_get_itotal(s->e, h->itotal);
}

int gbh_push_state(Hsolve *h)
{
    gbh_hstate *s = (gbh_hstate *)h->accel_state;
    if (!s) return 0;   /* no engine yet: gbh_init copies the host arrays */
    if (gbh_set_state(s->e, h->vm, h->chip, h->nconcs ? h->conc : NULL) != GBH_OK) {
        fprintf(stderr, "gbh_push_state %s: %s\n", h->name, gbh_last_error());
        return -1;
    }
    return 0;
}

void gbh_cleanup(void)
{
    int k;
    for (k = 0; k < gbh_nreg; k++) {
        Hsolve *h = gbh_registry[k];
        gbh_hstate *s = (gbh_hstate *)h->accel_state;
        if (!s) continue;
        gbh_destroy(s->e);
        free(s->in_msg);
        free(s->in_vals);
        free(s);
        h->accel_state = NULL;
    }
    gbh_nreg = 0;
}
