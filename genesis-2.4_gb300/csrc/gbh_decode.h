// gbh_decode.h -- host-side decoding of reference hsolve arrays into the
// engine's per-neuron micro-programs and tile layout.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>
#include "gbhsolve.h"
#include "gbh_internal.h"

namespace gbh {

enum FieldKind { FS_CHIP = 0, FS_GIV = 1, FS_CONST = 2, FS_CCHIP = 3, FS_WDT = 4, FS_COV0 = 5, FS_BUFV = 6 };

struct FieldSrc {
    int kind;
    int64_t idx;     // chip / givals / concchip index within the solver
    bool state;      // written back on sync (gate states, synchan X/Y)
};

// One neuron = one tree of one solver (a solver with symmetric compartments:
// the whole solver, its elimination program run as written).
struct Neuron {
    int solver = 0;
    int row0 = 0, nrows = 0;
    int table_set = 0, crank = 0, c5 = 0, interp = 1;
    std::vector<int> prog;        // micro-ops of all its compartments
    std::vector<int> pool_prog;   // 0-terminated
    std::vector<FieldSrc> fsrc;
    std::vector<double> fval;
    std::vector<int> iops;        // ops index backing each int row
    std::vector<int> ival;
    std::vector<int> pool_conc;   // solver conc index of each pool row
    std::vector<int64_t> giv_ref; // solver givals index of each givals row
    std::vector<int> syn_op;      // solver ops index of each synchan row
    std::vector<int> stab_pos;    // prog positions holding a stablist index
    std::vector<int> parent;      // per slot
    std::vector<double> A, B, C;  // per slot
    std::vector<int> ridx;        // per slot: ravals index of A, B, C (-1: none)
    std::vector<int> sym;         // symmetric compartments: SymOp triples (empty: a tree)
    std::vector<double> rav;      // symmetric compartments: the solver's ravals
    int spike_op = -1;
    bool has_cd = false;          // diffusion systems: codiag/coresult rows in use
    int nscratch = 0;             // scratch rows of its diffusion solves
    int nitot = 0;                // storemode: itotal rows (the solver's nelm_names)
    std::string key;              // grouping signature
};

struct Decoded {
    std::vector<Neuron> neurons;
    std::vector<double> stablist;             // deduplicated synchan constants (4 per entry)
    std::vector<int> solver_first_neuron;  // [nsolvers+1]
};

// Decodes every solver of the batch; returns GBH_OK or an error code with
// *err filled (solver, row, opcode, position, message).
int decode_batch(const gbh_batch_desc *d, Decoded &out, gbh_error *err);

}  // namespace gbh
