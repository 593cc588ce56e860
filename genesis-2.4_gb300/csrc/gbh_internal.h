// gbh_internal.h -- shared definitions between the host decoder and the
// device kernels of the GB300 hsolve engine.
#pragma once
#include <stdint.h>

namespace gbh {

// ---- reference opcode values (genesis/src/hines/hines_defs.h:120-222) ----
enum RefOp {
    R_TABCURR = 0, R_COMPT = 100, R_FCOMPT = 101, R_LCOMPT = 102, R_SPIKE = 200,
    R_ELMMPUMP = 500, R_CONC_VAL = 1000, R_NERNST = 2000, R_GHK = 2010, R_CHAN = 3000,
    R_CHAN_EK = 3001, R_SAME_GHK = 3002, R_DO_TABGHK = 3003, R_ADD_CURR = 3200,
    R_FLUX = 3300, R_SCALE_FLUX = 3301, R_STORE_ALLI = 3501, R_STORE_ALLC = 3502,
    R_IPOL1V = 4001, R_IPOL1C = 4002, R_IPOL2V = 4003, R_IPOL2C = 4004, R_SYN2 = 4100,
    R_SYN3 = 4101, R_MGBLOCK = 4200, R_NEWVOLT = 5100, R_NEWCONC1 = 5110,
    R_NEWCONC2 = 5111, R_DOMAIN = 5112,
    R_CONC = 10100, R_FCONC = 10101, R_LCONC = 10102, R_FLUXCONC = 10103,
    R_CACONC = 10200, R_LCACONC = 10202, R_TAUPUMP = 11000, R_CTAUPUMP = 11001, R_MMPUMP = 11010,
    R_HILLPUMP = 11011, R_PHILLPUMP = 11012, R_BUFFER = 12000, R_POOL = 12100
};
enum RefFunc { F_ELIM = 0, F_SET_DIAG = 1, F_SKIP_DIAG = 2, F_FASTSIB = 3, F_COPY = 4,
               F_SIB = 5, F_CALC = 6, F_FINISH = 7 };

// ---- engine micro-ops: one compartment program is a list of these ----
// Operands named f* are field rows of the tile's parameter block; p* are pool
// rows; i* are rows of the integer-state block; g* are givals rows (or -1).
enum MicroOp {
    M_BEGIN = 1,     // fEmRm fInject fRm gIleak                       (row start)
    M_NEWVOLT,       //                                                 (locate V)
    M_CONCVAL,       // pConc                                           (select pool, flux=0)
    M_DOMAIN,        // fScale                                          (locate C at scale*Ik)
    M_NEWCONC2,      // pConc                                           (save C1, locate C2)
    M_NEWCONC1,      //                                                 (locate C at conc[sel])
    M_SPIKE,         // fThresh iCounter iRefract                       (spike detect)
    M_ELMMPUMP,      // fKd fVmax fDiag gOut                            (electrogenic pump)
    M_FLUX,          //                                                 (flux[sel] += Ik)
    M_SCALE_FLUX,    // fScale
    M_GHK,           // fZFRT fZF fGmax                                 (GHK + SAME_GHK)
    M_SAME_GHK,      // fGmax
    M_DO_TABGHK,     //
    M_NERNST,        // fConst fGmax
    M_CHAN,          // fEk fGmax                                       (CHAN_EK / CHAN with Ek)
    M_CHAN_G,        // fGmax                                           (CHAN keeping Ek)
    M_GATE,          // kind col power fState                           (IPOL* + DOPOWER)
    M_SYN,           // fFreq stab sRow fX fY fWdt                      (SYN2/SYN3)
    M_MGBLOCK,       // fKA fKBinv fCMg gOut                            (after M_SYN)
    M_ADDCURR,       // gOut
    M_STORE,         // kind(0 I, 1 G) k                                 (itotal[k] += Ik / Gk)
    M_END,           // fTbyc fDiag gIm
    M_ITLEAK         // fEmRm fRm k                                      (itotal[k] += leak current)
};
enum GateKind { GK_1V = 0, GK_1C = 1, GK_2V = 2, GK_2C = 3 };
// Pool-phase micro-ops (do_h4_conc_chip_update, hines_conc_chip.c:59-221, and
// do_h_conc_solve, hines_conc.c:39-396). Operands: p* pool (conc) rows,
// f* field rows, s a compartment slot; `ix` is the current conc of a group
// and `res` its running result.
enum PoolOp {
    PO_CACONC = 1,    // p fBase fItau fDtB              Ca_concen
    PO_GRP = 2,       // p                               ix = p, res = 0 (FCONC/CONC)
    PO_STORE = 3,     //                                 coresult[ix] = res
    PO_FLUXCONC = 4,  // f0 f1                           res += f0 + flux[ix] f1
    PO_CTAU = 5,      // f0 f1                           res += f0, codiag[ix] += f1
    PO_TAU = 6,       // s f0 f1 f2 f3 f4                voltage-dependent tau pump
    PO_MM = 7,        // f0 f1                           codiag[ix] += f0 / (c[ix] + f1)
    PO_HILL = 8,      // h f0 f1                         Hill pump on ix
    PO_PHILL = 9,     // h p f0 f1 f2                    Hill pump from shell p into ix
    PO_BUFFER = 10,   // p f0 f1 f2                      pool buffer p of ix
    PO_POOL = 11,     //                                 c[ix] += res
    PO_DIFF = 12      // ms w nfix crank sbase nq nb, ms*w rows p, nq rows f, nb rows f
};

// Elimination program of a solver with symmetric compartments: the funcs[]
// tokens of do_euler_hsolve / do_crank_hsolve (hines_solve.c:140-296) as
// triples {token, a, b} with the ravals cursor resolved into an index.
//   forward:  SY_ELIM   row ra   temp = rav[ra] / diag[row]; diag -= rav[ra+1] temp;
//                                rhs -= rhs[row] temp
//             SY_SET / SY_SKIP   store the current row, move on by 1 / 2 rows
//             SY_FASTSIB dst ra  rav[dst] -= rav[ra] temp
//             SY_COPY  dst ra    rav[dst] = rav[ra]
//             SY_SIB   src dst   rav[dst] -= rav[src] temp
//   backward: SY_ELIM  row ra    rhs -= rav[ra] x[row]
//             SY_CALC            solve the current row, move down one row
//             SY_SIB   src row   rhs -= rav[src] x[row]
//   SY_FINISH ends each pass.
enum SymOp { SY_ELIM = 0, SY_SET = 1, SY_SKIP = 2, SY_FASTSIB = 3, SY_COPY = 4, SY_SIB = 5, SY_CALC = 6,
             SY_FINISH = 7 };

// Lanes per tile: one neuron per lane of a warp.
constexpr int LANES = 32;

struct TableGeom {
    int ncols, xdivs, ydivs, pad;
    double xmin, invdx, ymin, invdy;
    int64_t tab_off;   // offset into the table pool (doubles / floats)
    int64_t xv_off;    // offset into the value pool (xvals)
    int64_t yv_off;    // offset into the value pool (yvals), -1 if none
    // double-float copies of the axis constants for the mixed-precision kernel
    float xmin_hi, xmin_lo, invdx_hi, invdx_lo;
    float ymin_hi, ymin_lo, invdy_hi, invdy_lo;
};

struct TileType {
    int nslots;      // compartments per neuron
    int nfields;     // double rows in the parameter block
    int nints;       // int rows
    int npools;      // conc rows
    int ngiv;        // givals rows
    int prog_off;    // offset of slot 0's program in the micro-op pool
    int pool_off;    // offset of the pool program
    int table_set;
    int crank;       // 1 = Crank-Nicolson
    int chanmode5;
    int interp;      // calcmode
    int has_spike;
    int nsyn;        // synchan rows
    int has_cd;      // keeps codiag rows (diffusion systems): ELMMPUMP adds to them
    int nscratch;    // per-lane scratch rows of the diffusion solves
    int wide;        // one neuron per tile, its compartments across a block's threads
    int wide_off;    // wide: prog-pool offset of [slot program offsets | previous NEWVOLT slot |
                     //        previous NEWCONC1 slot | NEWCONC1 conc row], nslots each
    int sym;         // symmetric compartments: the solver's funcs program runs as written
    int sym_off;     // sym: prog-pool offset of its decoded triples (SymOp)
    int nrav;        // sym: ravals rows (rewritten during each step, as in the reference)
    int nitot;       // storemode: itotal rows, zeroed at the start of every step
    int stack;       // lane-mapped with the stack elimination (k_stack*): every neuron's rows are
                     // a post-order of its tree (each subtree contiguous, its root last)
    int scap;        // stack: shared-memory doubles per lane its neurons need
    int pf_off;      // stack: prog-pool offset of each slot's [first, last] field row (prefetch)
    int nstatic;     // stack: rows [0, nstatic) are passive and so is every row below them in their
                     // trees (the first non-passive slot; post-order keeps subtrees below their roots):
                     // their diagonals, reciprocals and coupling factors are the same every step
    int np1;         // stack: no row of any of its neurons has more than one stacked child (binary
                     // trees): the forward sweep pops at most one entry per row, without a loop
    int slots;       // stack, np1: every row's stack entries are below 32 and packed in its flags
                     // (FL_SLOT_*), so the sweeps index the stack without a running top
};

// Per-row flags of the stack elimination (DevView::ltop, topo rows, one word
// per lane). Forward, rows ascending: a row's last child is the row before
// it, whose contribution is carried in registers; its other children's
// contributions wait on a per-lane stack (they are its top FL_NPOP entries,
// in ascending row order). Backward, rows descending: the solution of the
// row after is in a register; a row whose parent is further away reads the
// parent's solution from a per-lane stack of branch points.
// Rows above the static ones (TileType::nstatic) that a second warp of a
// stack tile computes in shared memory while the first sweeps the static rows
constexpr int kSplitRows = 8;

enum StackFlag {
    FL_NPOP = 0xff,          // stack entries to apply: children other than the last
    FL_CARRY_IN = 1 << 8,    // the previous row is this row's last child
    FL_PARENT = 1 << 9,      // the row has a parent
    FL_CARRY_OUT = 1 << 10,  // the parent is the next row
    FL_PUSH = 1 << 11,       // the parent is further away: push the contribution
    FL_XLOAD = 1 << 12,      // backward: the parent's solution is on the stack top
    FL_XPOP = 1 << 13,       // backward: the last reader of that entry (the parent's first child)
    FL_XPUSH = 1 << 14,      // backward: two or more children read this row's solution later
    FL_PD = 1 << 15          // a row below nstatic whose parent is at or above it: the parent's
                             // forward step needs this row's diagonal contribution
};
// TileType::slots: bits 16-20 the forward entry (the stack depth after the
// row's pops: its stacked child is read there and its own contribution
// written there), 21-25 the backward entry its parent's solution is read
// from, 26-30 the backward entry its own solution is written to.
constexpr int FL_SLOT_F = 16, FL_SLOT_R = 21, FL_SLOT_W = 26;

struct Tile {
    int type;
    int nlanes;      // active lanes
    int64_t fld;     // row offsets (x32 elements) into the pools below
    int64_t topo;    // parent / A / B / C rows (nslots each)
    int64_t ints;
    int64_t pools;
    int64_t giv;
    int64_t vm;      // nslots rows
    int64_t syn;     // event-ring rows (nsyn * ring_len)
    int64_t scr;     // diffusion scratch rows (nscratch)
    int64_t wtop;    // wide: offset into DevView::wtop of its elimination schedule
    int64_t rav;     // sym: ravals rows (nrav)
    int64_t itot;    // storemode: itotal rows (nitot)
    int64_t first_neuron; // global neuron index of lane 0
};

// Device status word bits
// (bit 2 is unused: an event ring slot is consumed ring_len - 1 steps before
// it is reused, every delay being shorter than the ring, so it cannot overflow)
enum Status { ST_OK = 0, ST_BAD_OP = 1, ST_SMEM = 4 /* launched with too little shared memory */,
              ST_BARRIER = 8 /* a grid barrier wait ran out */,
              ST_NONFINITE = 16 /* a neuron's Vm became NaN, infinite or beyond 1e30 */ };

}  // namespace gbh
