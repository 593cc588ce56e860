/*
 * ref_cuda_host.c -- runs the reference's own CUDA backend
 * (genesis/src/hines/cuda/cuda_hsolve.c with cuda_backend.cu and
 * cuda_channel.cuh, compiled from the reference sources for sm_103a by
 * `make -C oracle cuda-ref`) on a solver given as the oracle's flat struct,
 * the way hines.c drives it under USE_CUDA (hines.c:224-268): per step
 * cuda_chip_update, then -- it returns 0 in its per-step mode -- the CPU
 * concentration update and Hines solve of the reference's own step code.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY: the reference's GPU arm, timed
 * beside the engine. Only the per-step mode is run: the multi-step mode's
 * tree kernel reads results[-2] for the first tree after its last row
 * (cuda_hines_tree_eliminate's CALC_RESULTS step, cuda_channel.cuh:498-501),
 * an out-of-bounds read this code does not start.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "hines_ext.h"
#include "hsolve_oracle.h"

extern int cuda_init(Hsolve *hsolve);
extern int cuda_chip_update(Hsolve *hsolve);
extern void cuda_cleanup(void);
extern int do_h4_conc_chip_update(Hsolve *);
extern void do_euler_hsolve(Hsolve *);
extern void do_crank_hsolve(Hsolve *);

/* the simulation clock GENESIS keeps (sim/sim_ext.h:38); cuda_chip_update
 * batches solvers by it */
double simulation_time;

static double now_ms(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

/* nsteps PROCESS steps of solver s through the reference's CUDA backend in
 * its per-step mode; wall_ms: host time of the steps (every step's copies,
 * kernel and CPU solve). Returns 0, or -1 when the backend refused the
 * solver or failed. */
int rch_perstep(orc_solver *s, int nsteps, double *wall_ms)
{
    Hsolve h;
    int i, rc = 0;
    double t0;
    memset(&h, 0, sizeof(h));
    h.name = "ref_cuda";
    h.ncompts = s->ncompts;
    h.chanmode = s->chanmode;
    h.calcmode = s->calcmode;
    h.ops = s->ops;       h.nops = s->nops;
    h.chip = s->chip;     h.nchips = s->nchips;
    h.funcs = s->funcs;   h.nfuncs = s->nfuncs;
    h.ravals = s->ravals; h.nravals = s->nravals;
    h.results = s->results;
    h.vm = s->vm;
    h.vmlast = s->vm + s->ncompts - 1;
    h.givals = s->givals; h.ngivals = s->ngivals;
    h.tablist = s->tablist; h.ncols = s->ncols; h.xdivs = s->xdivs;
    h.xmin = s->xmin;     h.invdx = s->invdx;   h.xvals = s->xvals;
    h.stablist = s->stablist;
    h.nconcs = s->nconcs; h.conc = s->conc;     h.flux = s->flux;
    h.nconcchips = s->nconcchips_used ? s->nconcchips : 0;
    h.concchip = s->concchip;
    h.nconcops = s->nconcops; h.concops = s->concops;
    h.childops = s->childops; h.childchips = s->childchips;
    h.dt = s->dt;
    if (cuda_init(&h) != 0) return -1;
    t0 = now_ms();
    for (i = 0; i < nsteps && rc == 0; i++) {
        int r;
        simulation_time = i * s->dt;
        r = cuda_chip_update(&h);
        if (r < 0) rc = -1;
        else if (r == 0) {   /* hines.c: the CPU finishes the step */
            if (h.nconcchips) do_h4_conc_chip_update(&h);
            if (s->crank) do_crank_hsolve(&h);
            else do_euler_hsolve(&h);
        }
    }
    *wall_ms = now_ms() - t0;
    cuda_cleanup();
    fflush(stdout);
    return rc;
}
