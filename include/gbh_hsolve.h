/*
 * gbh_hsolve.h -- hsolve-level C ABI of the GB300 step engine: many GENESIS
 * hsolve elements stepped together by one engine.
 *
 * Replaces the per-hsolve accelerator state and its process-wide registry in
 * the reference's CUDA backend (genesis/src/hines/cuda/cuda_hsolve.c:64-145:
 * cuda_state_register, cuda_batch_allowed, cuda_perstep_one), which the
 * one-hsolve-per-cell idiom (`call solver DUPLICATE`, e.g.
 * genesis/Scripts/VAnet2/VAnet2-batch.g:435-450) needs: thousands of
 * solvers, each called once per step by the scheduler. Here every registered
 * solver joins one batch engine; the first call of a step runs the whole
 * batch (one launch per step when the solvers share a program), later calls
 * in that step find it done. Unlike the reference, solvers with spike
 * detectors are batched too: their synapses onto synchans of solvers in the
 * batch are delivered on the device (gbh_synapses), so no spike needs GENESIS
 * messaging within a step; spikes also go to the host for targets outside
 * the batch (on_spike).
 *
 * GENESIS-free: the GENESIS side (genesis-2.4_gb300/adapter/
 * gbh_hsolve_adapter.c) fills a gbh_hs_solver from an Hsolve and its
 * messages. Arrays are borrowed: the engine copies them when the batch is
 * built, and gbh_hs_sync / per-step outputs write back into vm/chip/conc/ops.
 * Single caller thread, as GENESIS.
 */
#ifndef GBH_HSOLVE_H
#define GBH_HSOLVE_H

#include <stdint.h>

#include "gbhsolve.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One h_in_msgs input (hines_msgs.c:351-405): kind GBH_IN_SET / ADD / FLUX
 * as for gbh_register_inputs_typed, target index (chip[] or conc[]), factors,
 * and the message value, read through value(ctx) at each step. */
typedef struct gbh_hs_input {
    int kind;
    int64_t index;
    double sa, sb;
    double (*value)(void *ctx);
    void *ctx;
} gbh_hs_input;

/* One synapse from this solver's spike detector onto the synchan whose
 * SYN2_OP/SYN3_OP is ops[target_op] of the registered solver `target`
 * (an id returned by gbh_hs_register), with its weight and delay in steps
 * ((int)(delay/dt + 0.9), synchan.c:199-200). */
typedef struct gbh_hs_synapse {
    int target;
    int target_op;
    double weight;
    int delay_steps;
} gbh_hs_synapse;

typedef struct gbh_hs_solver {
    double dt;
    int method;                 /* 11 = Crank-Nicolson, else backward Euler */
    int chanmode, calcmode, storemode;
    int ncompts;
    int nops;       int *ops;
    int nchips;     double *chip;
    int nfuncs;     const int *funcs;
    int nravals;    const double *ravals;
    double *vm;
    int ngivals;    double *givals;
    int nstab;      const double *stablist;     /* sntab * 4 doubles */
    int nconcs;     double *conc;
    int nconcops;   const int *concops;
    int nconcchips; const double *concchip;
    gbh_tables tables;
    /* difshell systems (ndiffs > 0) */
    int ndiffs;
    const int *dconc, *nshells, *nshrows, *nshfix, *fbufval;
    int ncovals0;   const double *covals0;
    int nbufvals;   const double *bufvals;
    /* storemode: itotal[nelm_names] */
    int nelm_names; double *itotal;
    /* per-step inputs and outputs */
    int ninputs;    const gbh_hs_input *inputs;
    int has_outputs;            /* vm (and itotal) written back after every step (h_out_msgs) */
    /* spike detector: synapses in the batch, and a host call for every spike
     * when some of its targets are outside the batch */
    int nsynapses;  const gbh_hs_synapse *synapses;
    void (*on_spike)(void *ctx);
    void *spike_ctx;
} gbh_hs_solver;

/* Registers a solver (copies the struct, not the arrays). Returns its id
 * (>= 0; ids count up from 0 in registration order, which is taken as the
 * order the scheduler steps the solvers) or a negative error. The batch
 * engine is (re)built at the next new step; register every solver before
 * the first step (GENESIS: at RESET). */
int gbh_hs_register(const gbh_hs_solver *s);

/* Replaces solver id's synapses and spike callback (for synapses whose
 * targets are registered after the source, resolved before the first step).
 * The arrays are borrowed; the batch is rebuilt at the next new step. */
int gbh_hs_set_synapses(int id, int nsynapses, const gbh_hs_synapse *synapses, void (*on_spike)(void *ctx),
                        void *spike_ctx);

/* One PROCESS step of solver id, stamped with the simulation step number
 * (the same for every solver within a step, increasing between steps). The
 * first call with a new stamp reads every solver's inputs, runs the batch one
 * step, writes vm back for the solvers with outputs and calls on_spike; it
 * returns 1 (vm ready: skip the CPU conc update and solve) or a negative
 * error (setup errors are hard errors, there is no CPU fallback). */
int gbh_hs_step(int id, long long stamp);

/* Device -> the solver's vm, chip, conc, ops (and itotal). */
int gbh_hs_sync(int id);

/* The solver's host vm, chip, conc -> device (after RESTORE2, HPUT, RESET). */
int gbh_hs_push(int id);

/* Statistics of the batch engine (launches, steps, tiles). */
int gbh_hs_stats(gbh_stats *st);

/* Number of registered solvers. */
int gbh_hs_count(void);

/* Releases the batch engine and the registry. */
void gbh_hs_cleanup(void);

#ifdef __cplusplus
}
#endif
#endif /* GBH_HSOLVE_H */
