/*
 * hsolve_oracle.h -- CPU restatement of the GENESIS hsolve chanmode 4/5 step.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle that the GPU engine is checked
 * against; it is never linked into the engine library. Only the test suite,
 * the smoke check and the CPU-baseline leg of the benchmark load it.
 *
 * It operates on the same flat arrays the reference hsolve builds at SETUP
 * (ops[], chip[], funcs[], ravals[], tablist[], concops[], concchip[], ...)
 * and follows, function by function:
 *   orc_chip_update   <- do_chip_hh4_update / do_chip_hh4ni_update
 *                        (genesis/src/hines/hines_chip.c:78-602, instantiated
 *                        by hines_4chip.c:7-11 and hines_4nichip.c)
 *   orc_conc_update   <- do_h4_conc_chip_update (hines_conc_chip.c:59-221)
 *   orc_conc_solve    <- do_h_conc_solve (hines_conc.c:39-396)
 *   orc_solve         <- do_euler_hsolve / do_crank_hsolve (hines_solve.c:140-296)
 *   orc_process       <- HinesSolver PROCESS, chanmode 4/5 (hines.c:222-270)
 * Spike and synaptic-event hooks (h_dospike_event / h_dosynchan,
 * hines_conn.c:44-89) are routed to caller-supplied callbacks; the network
 * layer (orc_net_*) restates the synchan event queue (newconn/synchan.c:160-350)
 * with exact integer step arithmetic.
 *
 * Compile with -ffp-contract=off so that no multiply-add is fused, which is
 * what the reference's arithmetic order requires for bit-level comparisons.
 */
#ifndef HSOLVE_ORACLE_H
#define HSOLVE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_solver orc_solver;

/* Called when SPIKE_OP fires: (ctx, solver id). */
typedef void (*orc_spike_fn)(void *ctx, int solver_id);
/* Called when a SYN2/SYN3 countdown reaches zero: must add the due events'
 * contribution to chip[x_slot] and return the new countdown (steps to the next
 * pending event, or -1). (ctx, solver id, stablist index, child index, x_slot) */
typedef int (*orc_syn_fn)(void *ctx, int solver_id, int stab_index, int child_index,
                          int x_slot);

struct orc_solver {
    int id;
    int ncompts, nchips, nops, nfuncs, nravals, ngivals;
    int *ops;          /* [nops]   channel program (mutated: counters)      */
    double *chip;      /* [nchips] channel parameters and gate states        */
    int *funcs;        /* [nfuncs] elimination program                      */
    double *ravals;    /* [nravals] off-diagonal coefficients                */
    double *results;   /* [2*ncompts] (rhs, diag) pairs                      */
    double *vm;        /* [ncompts] membrane potential, Hines order          */
    double *givals;    /* [ngivals] computed variables (givals[0] unused)    */
    int chanmode;      /* 4 or 5                                              */
    int calcmode;      /* 1 = interpolate tables, 0 = nearest row            */
    int storemode;     /* 0, 1 (currents) or 2 (conductances) into itotal    */
    int crank;         /* 1 = Crank-Nicolson (method 11), 0 = backward Euler */
    double dt;
    /* voltage / concentration tables */
    int ncols, xdivs, ydivs;
    double xmin, invdx, ymin, invdy;
    double *tablist;   /* [(xdivs+1)*ncols] plus one padding row            */
    double *xvals;     /* [xdivs+2] (last entry is padding)                 */
    double *yvals;     /* [ydivs+2] or NULL                                 */
    double *stablist;  /* [4*sntab] synchan constants                        */
    /* concentrations */
    int nconcs;
    double *conc, *flux, *codiag, *coresult;
    int nconcchips, nconcops;
    int *concops;
    double *concchip;
    double *ovals;     /* givals cursor used by TAUPUMP_OP (may be NULL)     */
    /* diffusion systems (difshells and their buffers, do_h_conc_solve) */
    int ndiffs;
    int *dconc, *nshells, *nshrows, *nshfix, *fbufval;   /* [ndiffs] */
    double *covals0;   /* coupling / buffer-total terms, consumed in order  */
    double *bufvals;   /* 3 per buffer type: dt2*kBf, dt2*kBb, dt*kBb*Btot  */
    double *covals;    /* scratch: nshells*nshrows^2 of the largest system  */
    double *cores;     /* scratch: nshells*nshrows                          */
    int nconcchips_used;
    double *itotal;    /* [nelm_names] or NULL                               */
    int nelm_names;
    /* per-child op / chip offsets (hsolve->childops/childchips); only the
     * reference binding needs them, to locate a synchan's countdown slot */
    int *childops, *childchips;
    /* hooks */
    orc_spike_fn on_spike;
    orc_syn_fn on_syn;
    void *hook_ctx;
    /* diagnostics: first offending op index on error */
    int err_op;
};

/* Returns 0 on success, -1 on an unknown opcode (err_op is set). */
int orc_chip_update(orc_solver *s);
int orc_conc_update(orc_solver *s);
void orc_conc_solve(orc_solver *s);
void orc_solve(orc_solver *s);
/* One PROCESS step (chip update, conc update, elimination). */
int orc_process(orc_solver *s);
/* n PROCESS steps of one solver with no network; returns 0 or -1. */
int orc_run(orc_solver *s, int nsteps);
/* Runs nsteps steps and returns sum_n sum_j (vm[rows[j]] after step n+1 -
 * trace[n*ntargets + j])^2 in *loss: the loss of the engine's differentiated
 * form, for finite-difference checks. */
int orc_run_loss(orc_solver *s, int nsteps, int ntargets, const int *rows, const double *trace, double *loss);
/* nsteps steps recording vm[rows[j]] after each into out[i * nrows + j] and,
 * when tab_rows is not NULL, each compartment's voltage-table row into
 * tab_rows[i * ncompts + c]. */
int orc_run_trace(orc_solver *s, int nsteps, int nrows, const int *rows, double *out, int *tab_rows);

/* ---- network of solvers with spike -> synchan event delivery ---- */
typedef struct orc_net orc_net;
/*
 * Synapses are given in CSR over source solvers (the solver that owns the
 * spikegen). Each synapse targets (solver, child index of a synchan in that
 * solver), with a weight and a delay in steps. The synchan's stablist index
 * is taken from the target's ops[] at run time.
 */
orc_net *orc_net_create(int nsolvers, orc_solver **solvers, const int *syn_start,
                        const int *syn_target_solver, const int *syn_target_child,
                        const int *syn_target_op, const double *syn_weight,
                        const int *syn_delay_steps);
void orc_net_destroy(orc_net *n);
/* Runs nsteps; spikes counted per solver into spike_counts (may be NULL). */
int orc_net_run(orc_net *n, int nsteps, long long *spike_counts);
/* Replaces the per-solver PROCESS function (default orc_process); lets the
 * same event layer drive the reference's own step code. */
void orc_net_set_process(orc_net *n, int (*process)(orc_solver *));
/* Number of steps executed so far. */
long long orc_net_step_count(const orc_net *n);
void orc_net_deliver(orc_net *n, int count, const int *tgt_solver, const int *tgt_child, const int *tgt_op,
                     const double *w, const long long *fire_step);
/* Seeds SYN3_OP's generator as G_SEEDRNG does (sim/sim_random.c:212-222). */
void orc_seed_rng(long seed);

#ifdef __cplusplus
}
#endif
#endif
