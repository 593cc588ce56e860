/*
 * gbhsolve.h -- C ABI of the GB300 hsolve chanmode 4/5 step engine.
 *
 * Drop-in for the accelerator boundary of GENESIS hsolve (the reference's
 * genesis/src/hines/cuda/cuda_hsolve.h:22-25 and the array-level API of
 * genesis/src/hines/cuda/cuda_backend.cu:157-259, 396-444). The engine takes
 * the arrays the reference SETUP builds -- ops[], chip[], funcs[], ravals[],
 * tablist[], concops[], concchip[] ... -- for one or many hsolve elements,
 * copies them to the GPU, and advances them by whole PROCESS steps: channel
 * program, Ca pools and Hines elimination, all on the device. There is no CPU
 * fallback: an opcode or elimination token the engine does not implement is a
 * setup error naming the solver, compartment row and opcode.
 *
 * Plain pointers and sizes only; no GENESIS or CUDA types cross this header.
 * All arrays are read during gbh_create and not retained.
 */
#ifndef GBHSOLVE_H
#define GBHSOLVE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBH_ABI_VERSION 4

/* precision of gate/table arithmetic (elimination, Vm and Ca are always FP64) */
#define GBH_PREC_FP64 0
#define GBH_PREC_MIXED 1 /* gates, tables, interpolation in FP32 */

/* error codes */
#define GBH_OK 0
#define GBH_ERR_ARG -1        /* bad argument or size                        */
#define GBH_ERR_OPCODE -2     /* ops[]/concops[] opcode not implemented      */
#define GBH_ERR_FUNCS -3      /* funcs[] token not implemented / malformed   */
#define GBH_ERR_CUDA -4       /* CUDA runtime failure                        */
#define GBH_ERR_DEVICE -5     /* device-side status word (e.g. event ring)   */
#define GBH_ERR_UNSUPPORTED -6 /* model feature outside the engine's scope   */

typedef struct gbh_error {
    int code;
    int solver;     /* solver index, or -1                           */
    int row;        /* compartment row (Hines order), or -1          */
    int opcode;     /* offending ops[]/funcs[] value, or 0           */
    int position;   /* index into ops[]/funcs[]/concops[], or -1     */
    char message[256];
} gbh_error;

/*
 * One composite table set: hsolve->tablist/xvals/yvals and their geometry
 * (hines_struct.h:352-378). tablist has (xdivs+1)*ncols doubles; xvals has
 * xdivs+1 entries, yvals ydivs+1 (or NULL).
 */
typedef struct gbh_tables {
    int ncols, xdivs, ydivs;
    double xmin, invdx, ymin, invdy;
    const double *tablist;
    const double *xvals;
    const double *yvals;
} gbh_tables;

/*
 * A batch of hsolve elements, arrays concatenated solver after solver with
 * CSR offsets (length nsolvers+1). Per-solver arrays are exactly the
 * reference's: ops (hsolve->ops, nops), chip (nchips), funcs (nfuncs), ravals
 * (nravals), vm (ncompts), givals (ngivals, only the Rm entries are read),
 * stablist (4*sntab), conc (nconcs), concops (nconcops), concchip (nconcchips).
 * Empty ranges are allowed for concops/concchip/stablist/conc.
 */
typedef struct gbh_batch_desc {
    int abi_version;            /* GBH_ABI_VERSION */
    int nsolvers;
    double dt;                  /* hsolve->dt, common to the batch           */
    const int *method;          /* [nsolvers] 10 BEULER, 11 CRANK_INT        */
    const int *chanmode;        /* [nsolvers] 4 or 5                          */
    const int *calcmode;        /* [nsolvers] 1 interpolate, 0 nearest row    */
    const int *table_set;       /* [nsolvers] index into tables[]             */
    int ntables;
    const gbh_tables *tables;   /* [ntables]                                  */
    const int64_t *ops_start;    const int *ops;
    const int64_t *chip_start;   const double *chip;
    const int64_t *funcs_start;  const int *funcs;
    const int64_t *ravals_start; const double *ravals;
    const int64_t *vm_start;     const double *vm;
    const int64_t *givals_start; const double *givals;
    const int64_t *stab_start;   const double *stablist;
    const int64_t *conc_start;   const double *conc;
    const int64_t *concops_start;  const int *concops;
    const int64_t *concchip_start; const double *concchip;
    /* Concentration diffusion systems (difshells with buffers), solved by
     * do_h_conc_solve (hines_conc.c:39-396); diff_start NULL = none. Per
     * system: first conc (solver-local), shells, rows per shell (buffers +
     * the shell), fixed buffers among them, first bufvals entry
     * (hsolve->dconc, nshells, nshrows, nshfix, fbufval). covals0 and
     * bufvals as the reference's setup fills them (h_setup_conc_solve). */
    const int64_t *diff_start;   /* [nsolvers+1] */
    const int *dconc, *nshells, *nshrows, *nshfix, *fbufval;
    const int64_t *covals0_start; const double *covals0;
    const int64_t *bufvals_start; const double *bufvals;
    /* storemode (hsolve->storemode, hines_chip.c:134-166, 314-322): per
     * solver 0 (off), 1 (each compartment's leak current and the currents
     * of the STORE_ALLI_OP children) or 2 (the conductances of the
     * STORE_ALLC_OP children), summed over the solver every step into
     * itotal[nelm_names] (gbh_get_itotal). storemode NULL = 0 everywhere. */
    const int *storemode;          /* [nsolvers] */
    const int64_t *itotal_start;   /* [nsolvers+1]: nelm_names of each solver */
} gbh_batch_desc;

/*
 * Spike -> synchan connectivity between solvers of the batch (what
 * h_dospike_event / synchan EVENT / HSEVENT do through GENESIS messages,
 * hines_conn.c:44-108, newconn/synchan.c:160-313). CSR over source solvers
 * (the solver holding the spikegen). Each synapse targets the SYN2_OP whose
 * ops[] index (within the target solver) is target_op, with its own weight
 * and delay in steps ((int)(delay/dt + 0.9), synchan.c:199-200; 0 for a
 * delay under a tenth of a step). The events due in one step are summed into
 * the synchan's activation as weight/dt each, newest first, the order of the
 * reference's pending-event list (synchan.c:239-350): later spikes first,
 * then sources later in the solver order, then later synapses of a source.
 * A spike acts in step s + delay, one step later when the target's synapse
 * op runs before the source's spike op in the sequential order (an earlier
 * solver, or an earlier op of the same solver); with delay 0 the spike
 * detectors run in a pass of their own before each step.
 */
typedef struct gbh_synapses {
    int64_t nsynapses;
    const int64_t *src_start;  /* [nsolvers+1] */
    const int *target_solver;  /* [nsynapses]  */
    const int *target_op;      /* [nsynapses]  */
    const double *weight;      /* [nsynapses]  */
    const int *delay_steps;    /* [nsynapses]  */
} gbh_synapses;

/*
 * Synapses from sources outside this engine (cells simulated by other ranks
 * of a partitioned network). Sources are numbered by the caller (for
 * example by their global cell index); CSR over sources. Each synapse
 * targets the SYN2_OP (target_op, ops[] index within target_solver) of a
 * local solver. delay_steps is the effective delay: a spike of the source
 * during step s acts in step s + delay_steps (>= 1). With the reference's
 * sequential solver order this is (int)(delay/dt + 0.9), plus 1 when the
 * target's solver precedes the source's in the global order.
 */
typedef struct gbh_remote_synapses {
    int nsources;
    const int64_t *src_start;  /* [nsources+1] */
    const int *target_solver;  /* local solver */
    const int *target_op;
    const double *weight;
    const int *delay_steps;    /* >= 1: spikes are exchanged between steps */
    int64_t first_solver;      /* global index of this engine's solver 0 (the
                                  order events due in one step are summed in) */
} gbh_remote_synapses;

typedef struct gbh_options {
    int precision;       /* GBH_PREC_FP64 or GBH_PREC_MIXED                  */
    int steps_per_launch;/* 0 = autotune: gbh_create times trial steps on a saved
                            copy of the state for each candidate kernel variant
                            and steps-per-launch (networks: also cooperative
                            launches of K steps with a grid barrier per step),
                            restores the state and keeps the fastest; > 0 =
                            steps fused per launch; < 0 (networks) = -K steps
                            per cooperative launch                            */
    int warps_per_block; /* 0 = autotune                                      */
    int use_graph;       /* capture multi-launch runs in a CUDA graph         */
    int device;          /* CUDA device ordinal                                */
    int jit;             /* 0 = specialise each tile type's program at setup
                            (NVRTC) in three forms -- unrolled straight-line,
                            unrolled with the eliminated rows in shared memory,
                            and compact (runs of identical compartments looped)
                            -- and let the autotuner pick; 1 = unrolled form
                            only; 2 = compact form only; 3 = unrolled form with
                            shared-memory rows only; -1 = interpret the
                            programs                                          */
    int wide_min;        /* neurons with at least this many compartments run
                            one per warp, compartments across its threads;
                            the other large neurons run 32 per warp, one per
                            lane, with the stack elimination. 0 = chosen by
                            trial at creation (candidates 32, 64, 128, never:
                            an interpreted engine per candidate times a few
                            steps; with jit 0 the chosen mapping is also timed
                            specialised, and specialisation is turned off
                            when it is slower); < 0 = never
                            (gbh_loss_gradient needs it)                      */
} gbh_options;

typedef struct gbh_stats {
    int64_t steps;
    double device_ms;          /* device time of gbh_run calls (CUDA events) */
    int64_t compartments;
    int64_t tiles;             /* warps of 32 neurons                          */
    int64_t launches;          /* kernel launches issued                       */
    double bytes_per_step;     /* algorithmic bytes streamed per step          */
    int steps_per_launch;
    int warps_per_block;
    int precision;
    int jit_kernels;           /* programs specialised and compiled at setup   */
    int jit_min_blocks;        /* resident 4-warp blocks per SM the chosen
                                  specialised variant was compiled for        */
    double grad_forward_ms;    /* last gbh_loss_gradient: checkpointed forward
                                  pass (device time, CUDA events)             */
    double grad_reverse_ms;    /* last gbh_loss_gradient: segment recomputation
                                  + adjoint steps (device time)               */
    int jit_compact;           /* form of the chosen specialised variant:
                                  0 unrolled, 1 compact (looped), 2 unrolled
                                  with its rows in shared memory              */
    int cooperative;           /* network steps run K per cooperative launch
                                  with a grid barrier between steps           */
    int64_t wide_tiles;        /* tiles holding one neuron across a warp's
                                  threads (level-by-level elimination)        */
    int64_t stack_tiles;       /* tiles of 32 large neurons, one per lane,
                                  eliminated with per-lane stacks             */
    int64_t grad_kept_steps;   /* last gbh_loss_gradient: 1 if every step's
                                  state stayed in device memory (no segment
                                  recomputed), 0 if segments were recomputed
                                  from checkpoints                            */
} gbh_stats;

typedef struct gbh_engine gbh_engine;

/* Builds the device engine; returns NULL and fills *err on failure. */
gbh_engine *gbh_create(const gbh_batch_desc *desc, const gbh_synapses *syn,
                       const gbh_options *opt, gbh_error *err);

/*
 * gbh_create with synapses from remote sources (a partitioned network: one
 * engine per rank). The caller exchanges spikes between steps:
 *   gbh_run(e, 1);
 *   gbh_get_spiked(e, mine);          -- local solvers that spiked
 *   (all-gather the bitmaps across ranks)
 *   gbh_deliver_remote(e, theirs);    -- remote sources that spiked
 * No counterpart in the reference (PGENESIS exchanges through messages).
 */
gbh_engine *gbh_create_dist(const gbh_batch_desc *desc, const gbh_synapses *syn,
                            const gbh_remote_synapses *remote, const gbh_options *opt, gbh_error *err);

/* Local solvers with a spikegen that spiked since the previous call, one bit
 * per solver (bit i of byte i/8), ceil(nsolvers/8) bytes; clears the record. */
int gbh_get_spiked(gbh_engine *e, uint8_t *solver_bits);

/* Remote sources that spiked during the step just run, one bit per source
 * (ceil(nsources/8) bytes, host memory): their synapses' events are placed
 * for step (step just run) + delay_steps. Call before the next step. */
int gbh_deliver_remote(gbh_engine *e, const uint8_t *source_bits);

/*
 * Runs only the host-side decoder (no GPU needed): checks that every opcode
 * and elimination token is implemented and reports the layout the engine
 * would use. Returns GBH_OK or the error gbh_create would return.
 * n_neurons / n_tiles / n_types may be NULL.
 */
int gbh_validate(const gbh_batch_desc *desc, gbh_error *err, int64_t *n_neurons, int64_t *n_types);

/*
 * Diagnostics: writes the CUDA source the engine generates for tile type
 * type_index (neurons sharing one program) into buf (NUL-terminated,
 * truncated to buflen). Returns the full source length, or a negative error.
 * compact: 0 unrolled form, 1 compact (looped) form, 2 unrolled form with its
 * rows in shared memory. Needs no GPU.
 */
int64_t gbh_jit_source(const gbh_batch_desc *desc, int precision, int type_index, int compact, char *buf,
                       int64_t buflen);

/* Advances every solver by nsteps PROCESS steps. Returns GBH_OK or an error. */
int gbh_run(gbh_engine *e, int nsteps);

/* Same, on a caller-owned CUDA stream (cudaStream_t passed as void*; NULL =
 * the engine's own stream, the one gbh_run uses). Returns once queued. */
int gbh_run_async(gbh_engine *e, int nsteps, void *stream);

/*
 * Copies state back into reference-layout arrays (concatenated like the
 * batch desc; any pointer may be NULL to skip): vm, chip (gate states and
 * synchan X/Y updated in place over a copy of the original chip), conc,
 * and ops (spike refractory counters and synchan countdowns).
 */
int gbh_get_state(gbh_engine *e, double *vm, double *chip, double *conc, int *ops);

/* Writes vm / chip / conc back into the engine (HPUT / RESTORE2 path). */
int gbh_set_state(gbh_engine *e, const double *vm, const double *chip, const double *conc);

/*
 * Copies the givals of the last completed step into a reference-layout array
 * (the kernel records them on the final step of a gbh_run when enabled).
 */
int gbh_enable_givals(gbh_engine *e, int enable);
int gbh_get_givals(gbh_engine *e, double *givals);

/*
 * Copies hsolve->itotal of every storemode solver after the last completed
 * step (layout itotal_start; solvers with storemode 0 are left untouched).
 * Replaces the host reads of hsolve->itotal (hines.c:285-290, element field
 * `itotal`).
 */
int gbh_get_itotal(gbh_engine *e, double *itotal);

/*
 * Per-step inputs and outputs, the engine side of h_in_msgs / h_out_msgs
 * (genesis/src/hines/hines_msgs.c:351-405, 423-486).
 *
 * gbh_register_inputs names n chip[] entries (solver, index within that
 * solver's chip[]) that the caller rewrites between steps -- INJECT, BASE or
 * THRESH message targets. gbh_set_inputs_async copies n values from host
 * memory (pinned for full speed) and scatters them into the engine on the
 * given stream, ordered before the next gbh_run_async on that stream.
 *
 * gbh_register_outputs names n compartments (solver, Hines row) whose Vm the
 * caller records; gbh_get_outputs_async gathers them and copies n doubles to
 * host memory on the stream (complete after a stream synchronize). For these
 * two, stream NULL means the engine's own stream.
 */
int gbh_register_inputs(gbh_engine *e, int n, const int *solver, const int64_t *chip_index);

/*
 * The general form of h_in_msgs (hines_msgs.c:351-405): input i of kind
 *   GBH_IN_SET  (INJECT/BASE/THRESH)  chip[index] = v
 *   GBH_IN_ADD  (SYN2 messages)       chip[index] += v * sa * sb  when v > 1e-10
 *                                     (sa = stablist[nop+3]; sb = hsolve->dt for
 *                                     ACTIVATION messages into a synchan, else 1)
 *   GBH_IN_FLUX (FLUX messages)       flux[index] = v  (index: conc index)
 * Inputs with the same target are applied in registration order, as the
 * reference walks its ininfo list. kind, sa, sb may be NULL (all SET, 1, 1).
 */
enum { GBH_IN_SET = 0, GBH_IN_ADD = 1, GBH_IN_FLUX = 2 };
int gbh_register_inputs_typed(gbh_engine *e, int n, const int *solver, const int *kind, const int64_t *index,
                              const double *sa, const double *sb);
int gbh_set_inputs_async(gbh_engine *e, const double *host_values, void *stream);
int gbh_register_outputs(gbh_engine *e, int n, const int *solver, const int *row);
int gbh_get_outputs_async(gbh_engine *e, double *host_values, void *stream);

/*
 * gbh_step_io -- one call per simulation step with host inputs and outputs,
 * pipelined: the registered inputs (host_in, n_in doubles, pinned memory
 * for overlap) are copied to the device on the engine's copy stream while
 * earlier work runs, scattered and stepped (nsteps steps) on `stream` (NULL
 * = the engine's stream), and the registered outputs are gathered and copied
 * to host_out on the copy stream while the next call's step runs. Device
 * staging is double-buffered: the buffers passed to a call may be reused,
 * and its host_out is complete, once the second following call has
 * returned, or after gbh_io_sync. Either pointer may be NULL. Results equal
 * gbh_set_inputs_async + gbh_run_async + gbh_get_outputs_async. No
 * counterpart in the reference (h_in_msgs / h_out_msgs run on the host).
 */
int gbh_step_io(gbh_engine *e, const double *host_in, double *host_out, int nsteps, void *stream);
int gbh_io_sync(gbh_engine *e);

/*
 * gbh_run_io -- nsteps steps with per-step host inputs and outputs streamed
 * in blocks: host_in holds nsteps rows of the registered inputs (row k is
 * applied before step k, as gbh_set_inputs_async), host_out receives nsteps
 * rows of the registered outputs (row k after step k). Each block of `block`
 * steps (0 = 16) is copied host->device in one transfer on a copy stream
 * while the previous block steps, and its outputs device->host in one
 * transfer while the next block steps; between two steps one kernel gathers
 * the outputs and scatters the next inputs. Staging is double-buffered on
 * the device (2 x block x (n_in + n_out) doubles). Either pointer may be
 * NULL. Returns when host_out is complete. Results equal nsteps rounds of
 * gbh_set_inputs_async + gbh_run_async(1) + gbh_get_outputs_async. Host
 * buffers should be pinned for the copies to overlap. Serves h_in_msgs /
 * h_out_msgs-style stimulus and recording for a whole run (the reference
 * runs both on the host every step, hines_msgs.c:351-486).
 */
int gbh_run_io(gbh_engine *e, const double *host_in, double *host_out, int nsteps, int block, void *stream);

/* Per-solver spike counts since creation (int64[nsolvers]). */
int gbh_get_spike_counts(gbh_engine *e, int64_t *counts);

int gbh_get_stats(const gbh_engine *e, gbh_stats *st);

/*
 * gbh_run_noalloc -- advance the engine by nsteps with no device allocation.
 *
 * No counterpart in the reference: its CUDA backend allocates per solver.
 * This exists for hosts that are not allowed to allocate device memory while
 * the simulation steps: a GENESIS process that shares the GPU with another
 * runtime which reserved the device memory at start-up (a caching pool sized
 * once, so a later cudaMalloc fails or steals from it), or a step loop with a
 * latency budget, where cudaMalloc/cudaFree may synchronise the whole device.
 * Results equal gbh_run's on the same engine, registered inputs included.
 *
 * The step kernel's per-step scratch -- the Ca flux rows, one double per Ca
 * pool per neuron slot, padded to 32 lanes -- comes from a fixed array of
 * GBH_NOALLOC_FLUX_MAX doubles (8 MiB) compiled into the library, which every
 * GPU that loads the library keeps until the process exits. Engines that need
 * more are rejected with GBH_ERR_ARG before anything is queued. The call
 * makes no cudaMalloc/cudaFree or other allocating call: it copies the
 * engine's flux rows (FLUX inputs set by gbh_set_inputs_async, flux carried
 * from the previous step) into the array, steps on it, and copies the rows
 * back, two device-to-device copies between buffers that already exist. The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the one array: calls that may overlap on the GPU (other
 * streams, other engines) race on it and must be serialised by the caller.
 * stream is a cudaStream_t passed as void* (NULL = the engine's own stream,
 * as for gbh_run_async); the call returns once the work is queued and leaves
 * the caller's current device as it found it. A device status word raised
 * by these steps (a non-finite Vm, an unimplemented micro-op) is reported by
 * the engine's next synchronous call (gbh_run).
 */
#define GBH_NOALLOC_FLUX_MAX (1 << 20)
int gbh_run_noalloc(gbh_engine *e, int nsteps, void *stream);

/*
 * gbh_loss_gradient -- differentiated form (FP64 engines only).
 *
 * No counterpart in the reference (GENESIS computes no gradients). From the
 * engine's current state it runs nsteps steps and returns
 *   loss = sum_n sum_j (Vm[solver_j, row_j] after step n+1 - trace[n][j])^2
 * for n = 0 .. nsteps-1, and its gradient with respect to every input of the
 * step (each output may be NULL):
 *   dchip   [total chip]   parameters read from chip[] (Em/Rm, inject, Ek,
 *                          gbar, dt/Cm, diagonal term) and the initial gate
 *                          states held there;
 *   dravals [total ravals] the elimination coefficients of every row;
 *   dvm0    [total vm]     the initial membrane potentials;
 * laid out like the arrays of the gbh_batch_desc given to gbh_create (solvers
 * concatenated through the *_start offsets). Entries the step does not read
 * are zero. The engine's own state is left unchanged.
 *
 * Method: hand-written adjoint (reverse-mode) kernels. A forward pass stores
 * Vm and the gate states every checkpoint_every steps; the reverse pass
 * recomputes each segment from its checkpoint, recording Vm, the
 * elimination's diagonals and right-hand sides, the solution and the gate
 * states of every step, and runs the transposed Hines sweep (reverse
 * elimination order) and the reverse of the gate updates and table
 * interpolations step by step back to the start, one segment of
 * checkpoint_every steps at a time. checkpoint_every <= 0: the forward pass
 * keeps every step's Vm and gate states when nsteps x (rows + gates)
 * doubles per neuron fit in 60% of the device memory left free beside the
 * tapes, and no segment is recomputed (segments of 100 steps); otherwise as
 * checkpoint_every = 100. The results are the same bits either way
 * (gbh_stats.grad_kept_steps says which ran). Device memory held during
 * the call: checkpoints ~ (nsteps / checkpoint_every) x (rows + gates)
 * doubles per neuron (nsteps x when every step is kept) and two tapes of
 * ~ checkpoint_every x (10 rows + 4 gates + channels) doubles per neuron.
 *
 * Supported programs (GBH_ERR_UNSUPPORTED otherwise): compartments with
 * voltage-tabulated channels (TABCHAN with IPOL1V gates of nonzero power,
 * leak through Em/Rm), chanmode 4 or 5, either calcmode, backward Euler or
 * Crank-Nicolson; no Ca pools, concentration gates, GHK, synchans, spike
 * detectors or output-only opcodes. Each target row may appear once.
 */
typedef struct gbh_loss_spec {
    int ntargets;
    const int *solver;      /* [ntargets] */
    const int *row;         /* [ntargets] Hines row within the solver */
    const double *trace;    /* [nsteps][ntargets] target Vm after each step, host memory */
} gbh_loss_spec;
int gbh_loss_gradient(gbh_engine *e, int nsteps, int checkpoint_every, const gbh_loss_spec *spec,
                      double *loss, double *dchip, double *dravals, double *dvm0);
void gbh_destroy(gbh_engine *e);

/* Static description of the last error on this thread (never NULL). */
const char *gbh_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* GBHSOLVE_H */
