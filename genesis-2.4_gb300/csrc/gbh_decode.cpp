// gbh_decode.cpp -- turns the reference hsolve arrays into per-neuron
// micro-programs.
//
// ops[] is walked exactly like do_chip_hh4_update walks it
// (genesis/src/hines/hines_chip.c:157-600): one compartment per
// FCOMPT/COMPT sentinel, chip[] and givals[] consumed sequentially. Every
// chip value a compartment reads becomes a field row of its neuron; the
// sequential state the reference carries from one compartment to the next
// (the Ek of a CHAN_OP, the selected conc of a CONC_VAL_OP) is resolved here
// into explicit operands, so the device sees self-contained programs.
//
// funcs[] is executed symbolically, as do_euler_hsolve runs it
// (hines_solve.c:223-296), to recover each row's parent and the three
// off-diagonal coefficients it uses, in the order the reference applies them.
#include "gbh_decode.h"

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <exception>
#include <functional>
#include <map>
#include <thread>
#include <unordered_map>

namespace gbh {

namespace {

struct Ctx {
    const gbh_batch_desc *d;
    gbh_error *err;
    int solver;
};

int fail(Ctx &c, int code, int row, int opcode, int64_t pos, const char *fmt, ...)
    __attribute__((format(printf, 6, 7)));

int fail(Ctx &c, int code, int row, int opcode, int64_t pos, const char *fmt, ...)
{
    if (c.err) {
        c.err->code = code;
        c.err->solver = c.solver;
        c.err->row = row;
        c.err->opcode = opcode;
        c.err->position = (int)pos;
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(c.err->message, sizeof(c.err->message), fmt, ap);
        va_end(ap);
    }
    return code;
}

// Per-neuron builder helpers ------------------------------------------------
struct NB {
    Neuron *n;
    std::unordered_map<int64_t, int> chip_field, cchip_field, giv_row, pool_row, int_row;
    std::map<double, int> const_field;
    int fld(int kind, int64_t idx, double val, bool state = false)
    {
        std::unordered_map<int64_t, int> *m = nullptr;
        if (kind == FS_CHIP) m = &chip_field;
        else if (kind == FS_CCHIP) m = &cchip_field;
        if (m) {
            auto it = m->find(idx);
            if (it != m->end()) {
                if (state) n->fsrc[it->second].state = true;
                return it->second;
            }
        }
        int f = (int)n->fsrc.size();
        n->fsrc.push_back({kind, idx, state});
        n->fval.push_back(val);
        if (m) (*m)[idx] = f;
        return f;
    }
    int cfield(double v)
    {
        auto it = const_field.find(v);
        if (it != const_field.end()) return it->second;
        int f = fld(FS_CONST, -1, v);
        const_field[v] = f;
        return f;
    }
    int giv(int64_t gi)
    {
        auto it = giv_row.find(gi);
        if (it != giv_row.end()) return it->second;
        int g = (int)n->giv_ref.size();
        n->giv_ref.push_back(gi);
        giv_row[gi] = g;
        return g;
    }
    // three consecutive givals rows starting at gi
    int giv3(int64_t gi)
    {
        int g = giv(gi);
        giv(gi + 1);
        giv(gi + 2);
        return g;
    }
    int pool(int k)
    {
        auto it = pool_row.find(k);
        if (it != pool_row.end()) return it->second;
        int p = (int)n->pool_conc.size();
        n->pool_conc.push_back(k);
        pool_row[k] = p;
        return p;
    }
    int introw(int opidx, int val)
    {
        auto it = int_row.find(opidx);
        if (it != int_row.end()) return it->second;
        int r = (int)n->iops.size();
        n->iops.push_back(opidx);
        n->ival.push_back(val);
        int_row[opidx] = r;
        return r;
    }
};

// funcs[] of symmetric compartments (h_funcs_init's symflag branch,
// hines_init.c:361-1273, emits COPY_ARRAY, FASTSIBARRAY_ELIM and
// SIBARRAY_ELIM): walked with the reference's operand counts and ravals
// cursor (hines_solve.c:223-296), every index checked against the rows and
// ravals, and written out as SymOp triples. `sym` is false when no such token
// occurs (the program is then a tree, handled by parse_funcs).
int parse_funcs_sym(Ctx &c, const int *f, int64_t nf, int64_t nra, int n, std::vector<int> &prog, bool &sym)
{
    prog.clear();
    sym = false;
    if (n < 2) return GBH_OK;
    int64_t fi = 0, ri = 0;
    int cur = 1;
    auto row_of = [&](int64_t at, int &row) -> bool {
        const int x = f[at];
        if (x < 0 || (x & 1) || x / 2 >= n) return false;
        row = x / 2;
        return true;
    };
    auto rav_ok = [&](int64_t k) { return k >= 0 && k < nra; };
    for (int pass = 0; pass < 2; ++pass) {
        for (;;) {
            if (fi >= nf) return fail(c, GBH_ERR_FUNCS, cur, 0, fi, "funcs[] ends inside an elimination pass");
            const int op = f[fi++];
            int a = 0, b = 0;
            if (op == F_ELIM) {
                if (fi >= nf || !row_of(fi, a) || !rav_ok(ri) || (pass == 0 && !rav_ok(ri + 1)))
                    return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "ELIM operand or ravals cursor out of range");
                ++fi;
                b = (int)ri;
                ri += pass == 0 ? 2 : 1;
            } else if (pass == 0 && (op == F_SET_DIAG || op == F_SKIP_DIAG)) {
                cur += op == F_SET_DIAG ? 1 : 2;
                if (cur >= n) return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "forward cursor past the last row");
            } else if (pass == 0 && (op == F_FASTSIB || op == F_COPY)) {
                if (fi >= nf || !rav_ok(f[fi]) || !rav_ok(ri))
                    return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "ravals index out of range");
                a = f[fi++];
                b = (int)ri++;
                sym = true;
            } else if (op == F_SIB) {
                if (fi + 1 >= nf || !rav_ok(f[fi]))
                    return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "SIBARRAY_ELIM operand out of range");
                a = f[fi];
                if (pass == 0) {
                    if (!rav_ok(f[fi + 1]))
                        return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "SIBARRAY_ELIM operand out of range");
                    b = f[fi + 1];
                } else if (!row_of(fi + 1, b)) {
                    return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "SIBARRAY_ELIM row out of range");
                }
                fi += 2;
                sym = true;
            } else if (pass == 1 && op == F_CALC) {
                if (cur < 0) return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "CALC_RESULTS below row 0");
                cur -= 1;
            } else if (op == F_FINISH) {
                prog.insert(prog.end(), {SY_FINISH, 0, 0});
                break;
            } else {
                return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "funcs token %d in the %s pass", op,
                            pass == 0 ? "forward" : "backward");
            }
            prog.insert(prog.end(), {op, a, b});
        }
        if (pass == 0) {
            if (cur != n - 1)
                return fail(c, GBH_ERR_FUNCS, cur, 0, fi, "forward pass ends at row %d, expected %d", cur, n - 1);
            cur = n - 2;
        } else if (cur != -1) {
            return fail(c, GBH_ERR_FUNCS, cur, 0, fi, "backward pass stops at row %d", cur);
        }
    }
    return GBH_OK;
}

// Symbolic execution of funcs[] (asymmetric compartments).
int parse_funcs(Ctx &c, const int *f, int64_t nf, const double *ra, int64_t nra, int n,
                std::vector<int> &parent, std::vector<double> &A, std::vector<double> &B,
                std::vector<double> &Cc, std::vector<int> &ridx)
{
    ridx.assign(3 * (size_t)n, -1);   // ravals index of A, B, C of each row
    parent.assign(n, -1);
    A.assign(n, 0.0);
    B.assign(n, 0.0);
    Cc.assign(n, 0.0);
    std::vector<int> fcount(n, 0), bcount(n, 0), lastkid(n, -1);
    int64_t fi = 0, ri = 0;
    if (n == 1) return GBH_OK;
    if (nf < 1) return fail(c, GBH_ERR_FUNCS, -1, 0, 0, "empty funcs[] for %d compartments", n);
    int cur = 1;
    for (;;) {
        if (fi >= nf) return fail(c, GBH_ERR_FUNCS, cur, 0, fi, "funcs[] ends inside the forward pass");
        const int op = f[fi++];
        if (op == F_ELIM) {
            if (fi >= nf || ri + 2 > nra)
                return fail(c, GBH_ERR_FUNCS, cur, op, fi, "truncated FORWARD_ELIM");
            const int kid = f[fi++] / 2;
            if (kid < 0 || kid >= cur || cur >= n)
                return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "FORWARD_ELIM row %d not below %d", kid, cur);
            if (parent[kid] != -1 || fcount[kid])
                return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "row %d eliminated twice", kid);
            if (kid <= lastkid[cur])
                return fail(c, GBH_ERR_UNSUPPORTED, cur, op, fi - 1,
                            "children of row %d are not in ascending row order", cur);
            lastkid[cur] = kid;
            parent[kid] = cur;
            ridx[3 * kid] = (int)ri;
            A[kid] = ra[ri++];
            ridx[3 * kid + 1] = (int)ri;
            B[kid] = ra[ri++];
            fcount[kid]++;
        } else if (op == F_SET_DIAG) {
            cur += 1;
        } else if (op == F_SKIP_DIAG) {
            cur += 2;
        } else if (op == F_FINISH) {
            break;
        } else {
            return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1,
                        "funcs token %d (symmetric-compartment elimination) is not implemented", op);
        }
        if (cur >= n) return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "forward cursor past the last row");
    }
    if (cur != n - 1)
        return fail(c, GBH_ERR_FUNCS, cur, 0, fi, "forward pass ends at row %d, expected %d", cur, n - 1);
    cur = n - 2;
    for (;;) {
        if (fi >= nf) return fail(c, GBH_ERR_FUNCS, cur, 0, fi, "funcs[] ends inside the backward pass");
        const int op = f[fi++];
        if (op == F_ELIM) {
            if (fi >= nf || ri + 1 > nra) return fail(c, GBH_ERR_FUNCS, cur, op, fi, "truncated BACKWARD_ELIM");
            const int p = f[fi++] / 2;
            if (cur < 0 || p != parent[cur] || bcount[cur])
                return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "BACKWARD_ELIM of row %d does not match its parent", cur);
            ridx[3 * cur + 2] = (int)ri;
            Cc[cur] = ra[ri++];
            bcount[cur]++;
        } else if (op == F_CALC) {
            if (cur < 0) return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "CALC_RESULTS below row 0");
            if (parent[cur] >= 0 && !bcount[cur])
                return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1, "row %d solved before its parent term", cur);
            cur -= 1;
        } else if (op == F_FINISH) {
            break;
        } else {
            return fail(c, GBH_ERR_FUNCS, cur, op, fi - 1,
                        "funcs token %d (symmetric-compartment elimination) is not implemented", op);
        }
    }
    if (cur != -1) return fail(c, GBH_ERR_FUNCS, cur, 0, fi, "backward pass stops at row %d", cur);
    return GBH_OK;
}

// Grouping key: everything the kernel's control flow depends on.
void make_key(Neuron &N)
{
    std::string key;
    auto put = [&](int v) { key.append(reinterpret_cast<const char *>(&v), sizeof(int)); };
    put(N.nrows); put(N.table_set); put(N.crank); put(N.c5); put(N.interp);
    put((int)N.fsrc.size()); put((int)N.iops.size()); put((int)N.pool_conc.size());
    put((int)N.giv_ref.size()); put((int)N.syn_op.size()); put(N.spike_op >= 0);
    put(N.has_cd); put(N.nscratch); put(N.nitot);
    put((int)N.prog.size());
    for (int v : N.prog) put(v);
    put((int)N.sym.size());
    for (int v : N.sym) put(v);
    put((int)N.rav.size());
    for (int v : N.pool_prog) put(v);
    N.key = std::move(key);
}

// Decodes solver si into neurons (appended); synchan constant sets go to
// stabs (deduplicated within it), their indices recorded in Neuron::stab_pos.
int decode_solver(const gbh_batch_desc *d, int si, std::vector<Neuron> &neurons, std::vector<double> &stabs,
                  gbh_error *err)
{
    Ctx c{d, err, si};
    {
        const int *ops = d->ops + d->ops_start[si];
        const int64_t nops = d->ops_start[si + 1] - d->ops_start[si];
        const double *chip = d->chip + d->chip_start[si];
        const int64_t nchip = d->chip_start[si + 1] - d->chip_start[si];
        const int n = (int)(d->vm_start[si + 1] - d->vm_start[si]);
        const double *giv = d->givals + d->givals_start[si];
        const int64_t ngiv = d->givals_start[si + 1] - d->givals_start[si];
        const int method = d->method[si], cm = d->chanmode[si], calc = d->calcmode[si];
        const int ts = d->table_set ? d->table_set[si] : 0;
        if (n <= 0) return fail(c, GBH_ERR_ARG, -1, 0, -1, "solver without compartments");
        if (cm != 4 && cm != 5) return fail(c, GBH_ERR_UNSUPPORTED, -1, cm, -1, "chanmode %d (engine runs 4 and 5)", cm);
        if (ts < 0 || ts >= d->ntables) return fail(c, GBH_ERR_ARG, -1, 0, -1, "table set %d out of range", ts);
        // storemode: itotal is a sum over the whole solver, accumulated in row
        // order (hines_chip.c:134-166, 314-322), so the solver stays one neuron
        const int smode = d->storemode ? d->storemode[si] : 0;
        const int64_t nelm = smode ? d->itotal_start[si + 1] - d->itotal_start[si] : 0;
        if (smode < 0 || smode > 2) return fail(c, GBH_ERR_ARG, -1, 0, -1, "storemode %d (0, 1 or 2)", smode);
        if (smode && (nelm < 1 || nelm > (1 << 20)))
            return fail(c, GBH_ERR_ARG, -1, 0, -1, "storemode %d with %lld itotal entries", smode, (long long)nelm);

        // elimination structure
        std::vector<int> parent, ridx, symprog;
        std::vector<double> A, B, Cc;
        const int *fs = d->funcs + d->funcs_start[si];
        const int64_t nfs = d->funcs_start[si + 1] - d->funcs_start[si];
        const int64_t nra = d->ravals_start[si + 1] - d->ravals_start[si];
        bool sym = false;
        int rc = parse_funcs_sym(c, fs, nfs, nra, n, symprog, sym);
        if (rc) return rc;
        if (sym) {   // the whole solver is one neuron; its rows are coupled beyond a tree
            parent.assign(n, -1);
            A.assign(n, 0.0);
            B.assign(n, 0.0);
            Cc.assign(n, 0.0);
            ridx.assign(3 * (size_t)n, -1);
        } else {
            rc = parse_funcs(c, fs, nfs, d->ravals + d->ravals_start[si], nra, n, parent, A, B, Cc, ridx);
            if (rc) return rc;
        }
        // trees: parents always have higher rows (Hines numbering)
        std::vector<int> tree(n, -1);
        std::vector<int> tmin, tmax;
        const bool whole = sym || smode;   // one neuron holds every row of the solver
        if (whole) {
            tree.assign(n, 0);
            tmin.push_back(0);
            tmax.push_back(n - 1);
        }
        for (int r = n - 1; r >= 0 && !whole; --r) {
            if (parent[r] < 0) {
                tree[r] = (int)tmin.size();
                tmin.push_back(r);
                tmax.push_back(r);
            } else {
                if (parent[r] <= r) return fail(c, GBH_ERR_FUNCS, r, 0, -1, "parent row not above child");
                tree[r] = tree[parent[r]];
                if (r < tmin[tree[r]]) tmin[tree[r]] = r;
            }
        }
        const int ntrees = (int)tmin.size();
        std::vector<int> cnt(ntrees, 0);
        for (int r = 0; r < n; ++r) cnt[tree[r]]++;
        // neurons in ascending row order
        std::vector<int> order(ntrees);
        for (int t = 0; t < ntrees; ++t) {
            if (tmax[t] - tmin[t] + 1 != cnt[t])
                return fail(c, GBH_ERR_UNSUPPORTED, tmin[t], 0, -1, "tree rows are not contiguous");
            order[ntrees - 1 - t] = t;  // trees were found from the top row down
        }
        std::vector<int> tree_neuron(ntrees);
        const int nbase = (int)neurons.size();
        for (int k = 0; k < ntrees; ++k) {
            Neuron nn;
            nn.solver = si;
            nn.row0 = tmin[order[k]];
            nn.nrows = cnt[order[k]];
            nn.table_set = ts;
            nn.crank = method == 11;
            nn.c5 = cm == 5;
            nn.interp = calc != 0;
            for (int r = nn.row0; r < nn.row0 + nn.nrows; ++r) {
                nn.parent.push_back(parent[r] < 0 ? -1 : parent[r] - nn.row0);
                nn.A.push_back(A[r]);
                nn.B.push_back(B[r]);
                nn.C.push_back(Cc[r]);
                for (int q = 0; q < 3; ++q) nn.ridx.push_back(ridx[3 * r + q]);
            }
            if (sym) {
                nn.sym = symprog;
                nn.rav.assign(d->ravals + d->ravals_start[si], d->ravals + d->ravals_start[si + 1]);
            }
            nn.nitot = (int)nelm;
            tree_neuron[order[k]] = nbase + k;
            neurons.push_back(std::move(nn));
        }
        std::vector<NB> nbs(ntrees);
        for (int k = 0; k < ntrees; ++k) nbs[k].n = &neurons[nbase + k];

        // ---- walk ops[] ----
        int64_t o = 0, ch = 0, g = 1;   // givals[0] is unused
        int row = 0;
        // sequential state carried by the reference between compartments
        int ek_kind = 0;         // 0 none, 1 static chip index, 2 dynamic in row ek_row
        int64_t ek_chip = -1;
        int ek_row = -1;
        int sel = -1, sel_row = -1;
        bool doghk = false;
        auto need = [&](int64_t k) { return o + k <= nops; };
        while (true) {
            if (o >= nops) return fail(c, GBH_ERR_OPCODE, row, 0, o, "ops[] ends without LCOMPT_OP");
            const int sentinel = ops[o++];
            if (sentinel == R_LCOMPT) break;
            if (sentinel != R_COMPT && sentinel != R_FCOMPT)
                return fail(c, GBH_ERR_OPCODE, row, sentinel, o - 1, "expected a compartment sentinel, found %d", sentinel);
            if (row >= n) return fail(c, GBH_ERR_OPCODE, row, sentinel, o - 1, "more compartments in ops[] than rows");
            NB &nb = nbs[tree_neuron[tree[row]] - nbase];
            Neuron &N = *nb.n;
            const int nrow0 = tree_neuron[tree[row]];
            std::vector<int> &P = N.prog;
            if (ch + 2 > nchip || g + 2 > ngiv) return fail(c, GBH_ERR_ARG, row, 0, o, "chip[]/givals[] too short");
            P.push_back(M_BEGIN);
            P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
            P.push_back(nb.fld(FS_CHIP, ch + 1, chip[ch + 1]));
            P.push_back(nb.fld(FS_GIV, g, giv[g]));
            P.push_back(nb.giv(g + 1));
            if (smode == 1) {   // itotal[0] += leak current (hines_chip.c:166)
                P.push_back(M_ITLEAK);
                P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                P.push_back(nb.fld(FS_GIV, g, giv[g]));
                P.push_back(0);
            }
            ch += 2;
            g += 2;
            auto sel_pool = [&](int64_t at) -> int {
                if (sel < 0 || tree[sel_row] != tree[row]) {
                    fail(c, GBH_ERR_UNSUPPORTED, row, ops[at], at,
                         "conc selected in another neuron (CONC_VAL_OP missing)");
                    return -1;
                }
                return nb.pool(sel);
            };
            while (o < nops && ops[o] > R_LCOMPT) {
                const int code = ops[o++];
                bool current = false;
                switch (code) {
                case R_NEWVOLT:
                    P.push_back(M_NEWVOLT);
                    break;
                case R_CONC_VAL: {
                    if (!need(1)) return fail(c, GBH_ERR_OPCODE, row, code, o, "truncated CONC_VAL_OP");
                    const int k = ops[o++];
                    const int64_t nconc = d->conc_start[si + 1] - d->conc_start[si];
                    if (k < 0 || k >= nconc) return fail(c, GBH_ERR_ARG, row, code, o - 1, "conc index %d out of range", k);
                    sel = k;
                    sel_row = row;
                    P.push_back(M_CONCVAL);
                    P.push_back(nb.pool(k));
                    break;
                }
                case R_DOMAIN:
                    // the concentration axis (yvals) exists only in a solver
                    // with concentrations (hines_chip.c:131-140); without one
                    // the reference's lookup reads through a NULL yvals
                    if (d->conc_start[si + 1] == d->conc_start[si])
                        return fail(c, GBH_ERR_ARG, row, code, o - 1, "DOMAIN_OP in a solver without concentrations");
                    P.push_back(M_DOMAIN);
                    P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                    ch++;
                    break;
                case R_NEWCONC2: {
                    if (!need(1)) return fail(c, GBH_ERR_OPCODE, row, code, o, "truncated NEWCONC2_OP");
                    const int k = ops[o++];
                    const int64_t nconc = d->conc_start[si + 1] - d->conc_start[si];
                    if (k < 0 || k >= nconc) return fail(c, GBH_ERR_ARG, row, code, o - 1, "conc index %d out of range", k);
                    P.push_back(M_NEWCONC2);
                    P.push_back(nb.pool(k));
                    break;
                }
                case R_NEWCONC1: {
                    int p = sel_pool(o - 1);
                    if (p < 0) return GBH_ERR_UNSUPPORTED;
                    P.push_back(M_NEWCONC1);
                    break;
                }
                case R_SPIKE: {
                    if (!need(2)) return fail(c, GBH_ERR_OPCODE, row, code, o, "truncated SPIKE_OP");
                    if (N.spike_op >= 0)
                        return fail(c, GBH_ERR_UNSUPPORTED, row, code, o - 1, "second spikegen in one neuron");
                    N.spike_op = (int)(o - 1);
                    P.push_back(M_SPIKE);
                    P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                    P.push_back(nb.introw((int)o, ops[o]));
                    P.push_back(nb.introw((int)o + 1, ops[o + 1]));
                    o += 2;
                    ch++;
                    break;
                }
                case R_ELMMPUMP: {
                    int p = sel_pool(o - 1);
                    if (p < 0) return GBH_ERR_UNSUPPORTED;
                    P.push_back(M_ELMMPUMP);
                    P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                    P.push_back(nb.fld(FS_CHIP, ch + 1, chip[ch + 1]));
                    P.push_back(nb.fld(FS_CHIP, ch + 2, chip[ch + 2]));
                    P.push_back(nb.giv(g));
                    ch += 3;
                    g += 1;
                    break;
                }
                case R_FLUX: {
                    int p = sel_pool(o - 1);
                    if (p < 0) return GBH_ERR_UNSUPPORTED;
                    P.push_back(M_FLUX);
                    break;
                }
                case R_SCALE_FLUX: {
                    int p = sel_pool(o - 1);
                    if (p < 0) return GBH_ERR_UNSUPPORTED;
                    P.push_back(M_SCALE_FLUX);
                    P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                    ch++;
                    break;
                }
                case R_STORE_ALLI:
                case R_STORE_ALLC: {   // itotal[k] += Ik / Gk (hines_chip.c:314-322)
                    if (!need(1)) return fail(c, GBH_ERR_OPCODE, row, code, o, "truncated STORE_ALL op");
                    const int k = ops[o++];
                    if (!smode)
                        return fail(c, GBH_ERR_ARG, row, code, o - 2, "STORE_ALL op in a solver without storemode");
                    if (k < 0 || k >= nelm)
                        return fail(c, GBH_ERR_ARG, row, code, o - 1, "itotal index %d out of range", k);
                    P.push_back(M_STORE);
                    P.push_back(code == R_STORE_ALLI ? 0 : 1);
                    P.push_back(k);
                    break;
                }
                case R_GHK:
                case R_NERNST: {
                    int p = sel_pool(o - 1);
                    if (p < 0) return GBH_ERR_UNSUPPORTED;
                    if (nb.pool(sel + 1) != p + 1)
                        return fail(c, GBH_ERR_UNSUPPORTED, row, code, o - 1, "Cin/Cout pools not adjacent");
                    if (code == R_GHK) {
                        P.push_back(M_GHK);
                        P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                        P.push_back(nb.fld(FS_CHIP, ch + 1, chip[ch + 1]));
                        P.push_back(nb.fld(FS_CHIP, ch + 2, chip[ch + 2]));
                        ch += 3;
                    } else {
                        P.push_back(M_NERNST);
                        P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                        P.push_back(nb.fld(FS_CHIP, ch + 1, chip[ch + 1]));
                        ch += 2;
                    }
                    ek_kind = 2;
                    ek_row = row;
                    current = true;
                    break;
                }
                case R_SAME_GHK:
                    P.push_back(M_SAME_GHK);
                    P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                    ch++;
                    current = true;
                    break;
                case R_DO_TABGHK:
                    P.push_back(M_DO_TABGHK);
                    doghk = true;
                    current = true;
                    break;
                case R_CHAN_EK:
                    P.push_back(M_CHAN);
                    P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                    P.push_back(nb.fld(FS_CHIP, ch + 1, chip[ch + 1]));
                    ek_kind = 1;
                    ek_chip = ch;
                    ch += 2;
                    current = true;
                    break;
                case R_CHAN:
                    if (ek_kind == 2 && ek_row == row) {
                        P.push_back(M_CHAN_G);
                    } else if (ek_kind == 1) {
                        P.push_back(M_CHAN);
                        P.push_back(nb.fld(FS_CHIP, ek_chip, d->chip[d->chip_start[si] + ek_chip]));
                    } else if (ek_kind == 0) {
                        P.push_back(M_CHAN);
                        P.push_back(nb.cfield(0.0));
                    } else {
                        return fail(c, GBH_ERR_UNSUPPORTED, row, code, o - 1,
                                    "CHAN_OP uses an Ek computed in another compartment");
                    }
                    P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                    ch++;
                    current = true;
                    break;
                default:
                    return fail(c, GBH_ERR_OPCODE, row, code, o - 1, "ops[] opcode %d is not implemented", code);
                }
                if (!current) continue;
                // conductance sub-program (hines_chip.c:412-590)
                for (;;) {
                    if (o >= nops) return fail(c, GBH_ERR_OPCODE, row, 0, o, "ops[] ends inside a channel");
                    const int k = ops[o++];
                    if (k == R_IPOL1V || k == R_IPOL1C || k == R_IPOL2V || k == R_IPOL2C) {
                        if (!need(2)) return fail(c, GBH_ERR_OPCODE, row, k, o, "truncated gate op");
                        const int kind = k == R_IPOL1V ? GK_1V : k == R_IPOL1C ? GK_1C : k == R_IPOL2V ? GK_2V : GK_2C;
                        const int col = ops[o++];
                        const int pw = ops[o++];
                        if (pw > 6 || pw < -6)
                            return fail(c, GBH_ERR_OPCODE, row, k, o - 1, "gate power %d outside -6..6", pw);
                        if ((kind == GK_1C || kind == GK_2C) && sel < 0 && kind == GK_1C) {
                            // C1 cursor comes from NEWCONC1/DOMAIN; nothing to check here
                        }
                        P.push_back(M_GATE);
                        P.push_back(kind);
                        P.push_back(col);
                        P.push_back(pw);
                        if (pw == 0) {
                            P.push_back(-1);
                            ek_kind = 2;
                            ek_row = row;
                            if (doghk) {
                                doghk = false;
                                break;
                            }
                            P.push_back(M_ADDCURR);
                            P.push_back(nb.giv3(g));
                            g += 3;
                            break;
                        }
                        P.push_back(nb.fld(FS_CHIP, ch, chip[ch], true));
                        ch++;
                        continue;
                    } else if (k >= R_SYN2) {
                        if (k != R_SYN2 && k != R_SYN3)
                            return fail(c, GBH_ERR_OPCODE, row, k, o - 1, "conductance opcode %d is not implemented", k);
                        if (!need(3)) return fail(c, GBH_ERR_OPCODE, row, k, o, "truncated SYN op");
                        int ffreq = -1;
                        if (k == R_SYN3) {
                            ffreq = nb.fld(FS_CHIP, ch, chip[ch]);
                            ch++;
                        }
                        const int stab = ops[o];
                        const int64_t nstab = d->stab_start[si + 1] - d->stab_start[si];
                        if (stab < 0 || stab + 4 > nstab)
                            return fail(c, GBH_ERR_ARG, row, k, o, "stablist index %d out of range", stab);
                        const int srow = (int)N.syn_op.size();
                        N.syn_op.push_back((int)(o - 1));
                        // identical constant sets share one entry, so identical cells
                        // of different solvers keep identical programs
                        const double *sv = d->stablist + d->stab_start[si] + stab;
                        int gstab = -1;
                        for (size_t q = 0; q + 4 <= stabs.size(); q += 4)
                            if (memcmp(&stabs[q], sv, 4 * sizeof(double)) == 0) { gstab = (int)q; break; }
                        if (gstab < 0) {
                            gstab = (int)stabs.size();
                            stabs.insert(stabs.end(), sv, sv + 4);
                        }
                        P.push_back(M_SYN);
                        P.push_back(ffreq);
                        N.stab_pos.push_back((int)P.size());
                        P.push_back(gstab);
                        P.push_back(srow);
                        P.push_back(nb.fld(FS_CHIP, ch, chip[ch], true));
                        P.push_back(nb.fld(FS_CHIP, ch + 1, chip[ch + 1], true));
                        P.push_back(nb.fld(FS_WDT, srow, 0.0));
                        ch += 2;
                        o += 3;
                        if (o < nops && ops[o] == R_MGBLOCK) {
                            o++;
                            P.push_back(M_MGBLOCK);
                            P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
                            P.push_back(nb.fld(FS_CHIP, ch + 1, chip[ch + 1]));
                            P.push_back(nb.fld(FS_CHIP, ch + 2, chip[ch + 2]));
                            P.push_back(nb.giv3(g));
                            ch += 3;
                            g += 3;
                        }
                        P.push_back(M_ADDCURR);
                        P.push_back(nb.giv3(g));
                        g += 3;
                        break;
                    } else if (k == R_ADD_CURR) {
                        P.push_back(M_ADDCURR);
                        P.push_back(nb.giv3(g));
                        g += 3;
                        break;
                    } else {
                        return fail(c, GBH_ERR_OPCODE, row, k, o - 1, "conductance opcode %d is not implemented", k);
                    }
                }
            }
            if (ch + 2 > nchip || g + 1 > ngiv) return fail(c, GBH_ERR_ARG, row, 0, o, "chip[]/givals[] too short");
            P.push_back(M_END);
            P.push_back(nb.fld(FS_CHIP, ch, chip[ch]));
            P.push_back(nb.fld(FS_CHIP, ch + 1, chip[ch + 1]));
            P.push_back(nb.giv(g));
            ch += 2;
            g += 1;
            (void)nrow0;
            row++;
        }
        if (row != n) return fail(c, GBH_ERR_OPCODE, row, 0, o, "ops[] has %d compartments for %d rows", row, n);

        // ---- concops (hines_conc_chip.c:59-221) and diffusion systems
        //      (hines_conc.c:39-396) ----
        {
            const int *cops = d->concops + d->concops_start[si];
            const int64_t ncops = d->concops_start[si + 1] - d->concops_start[si];
            const int64_t ccbase = d->concchip_start[si];
            const int64_t ncchip = d->concchip_start[si + 1] - ccbase;
            const int nconc = (int)(d->conc_start[si + 1] - d->conc_start[si]);
            const int64_t ds0 = d->diff_start ? d->diff_start[si] : 0;
            const int64_t ds1 = d->diff_start ? d->diff_start[si + 1] : 0;
            // Every conc belongs to one neuron: the one whose compartment program
            // reads it, or the one of a conc it is tied to (same diffusion system,
            // the shell a Hill pump draws from, the buffer of a pool).
            std::vector<int> uf(nconc), owner(nconc, -1);
            for (int k = 0; k < nconc; ++k) uf[k] = k;
            auto find = [&](int x) {
                while (uf[x] != x) x = uf[x] = uf[uf[x]];
                return x;
            };
            auto unite = [&](int a2, int b2) { uf[find(a2)] = find(b2); };
            auto claim = [&](int k, int nrn) -> bool {
                const int r = find(k);
                if (owner[r] >= 0 && owner[r] != nrn) return false;
                owner[r] = nrn;
                return true;
            };
            auto cidx = [&](int64_t at, int k) -> int {
                if (k < 0 || k >= nconc) {
                    fail(c, GBH_ERR_ARG, -1, cops[at], at, "conc index %d out of range", k);
                    return -1;
                }
                return k;
            };
            for (int64_t i = ds0; i < ds1; ++i) {
                const int c0 = d->dconc[i], ms = d->nshells[i], w = d->nshrows[i];
                if (ms < 2 || w < 1 || d->nshfix[i] < 0 || d->nshfix[i] > w - 1 || c0 < 0 ||
                    (int64_t)c0 + (int64_t)ms * w > nconc)
                    return fail(c, GBH_ERR_ARG, -1, 0, i - ds0,
                                "diffusion system %lld: %d shells x %d rows at conc %d do not fit",
                                (long long)(i - ds0), ms, w, c0);
                for (int j = 1; j < ms * w; ++j) unite(c0, c0 + j);
            }
            // first pass: ties between concs and the current group conc
            {
                int64_t co = 0;
                int ix = 0;
                while (co < ncops) {
                    const int op = cops[co++];
                    if (op == R_LCONC || op == R_LCACONC) break;
                    auto need2 = [&](int k) { return co + k <= ncops; };
                    if (op == R_CONC || op == R_FCONC || op == R_CACONC) {
                        if (!need2(1)) return fail(c, GBH_ERR_OPCODE, -1, op, co, "truncated concops");
                        const int k = cidx(co, cops[co]);
                        if (k < 0) return GBH_ERR_ARG;
                        if (op != R_CACONC) ix = k;
                        co++;
                    } else if (op == R_TAUPUMP) {
                        if (!need2(1)) return fail(c, GBH_ERR_OPCODE, -1, op, co, "truncated TAUPUMP_OP");
                        const int vr = cops[co++];
                        if (vr < 0 || vr >= n) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "vm index %d out of range", vr);
                        if (!claim(ix, tree_neuron[tree[vr]] - nbase))
                            return fail(c, GBH_ERR_UNSUPPORTED, vr, op, co - 1, "pump reads the Vm of another neuron");
                    } else if (op == R_HILLPUMP) {
                        co++;
                    } else if (op == R_PHILLPUMP) {
                        if (!need2(2)) return fail(c, GBH_ERR_OPCODE, -1, op, co, "truncated PHILLPUMP_OP");
                        const int k = cidx(co + 1, cops[co + 1]);
                        if (k < 0) return GBH_ERR_ARG;
                        unite(ix, k);
                        co += 2;
                    } else if (op == R_BUFFER) {
                        if (!need2(1)) return fail(c, GBH_ERR_OPCODE, -1, op, co, "truncated BUFFER_OP");
                        const int k = cidx(co, cops[co]);
                        if (k < 0) return GBH_ERR_ARG;
                        unite(ix, k);
                        co++;
                    } else if (op != R_FLUXCONC && op != R_CTAUPUMP && op != R_MMPUMP && op != R_POOL) {
                        return fail(c, GBH_ERR_OPCODE, -1, op, co - 1, "concops opcode %d is not implemented", op);
                    }
                }
            }
            for (int k = 0; k < ntrees; ++k)
                for (int pc : nbs[k].n->pool_conc)
                    if (!claim(pc, k))
                        return fail(c, GBH_ERR_UNSUPPORTED, -1, 0, pc,
                                    "conc %d is tied to concentrations of two neurons", pc);
            auto owner_of = [&](int k) -> int {
                const int r = find(k);
                if (owner[r] < 0 && ntrees == 1) owner[r] = 0;
                return owner[r];
            };
            // second pass: micro-ops into the owning neuron's pool program
            int64_t co = 0, cc = 0;
            int ix = 0, grp = -1;   // current group conc and its owner
            auto chipf = [&](NB &nb, int64_t k) { return nb.fld(FS_CCHIP, k, d->concchip[ccbase + k]); };
            auto need_chips = [&](int k) { return cc + k <= ncchip; };
            auto open_group = [&](int k) -> int {
                const int o2 = owner_of(k);
                if (o2 < 0) return -1;
                NB &nb = nbs[o2];
                nb.n->pool_prog.push_back(PO_GRP);
                nb.n->pool_prog.push_back(nb.pool(k));
                nb.n->has_cd = true;
                return o2;
            };
            auto close_group = [&](bool store) {
                if (grp >= 0 && store) nbs[grp].n->pool_prog.push_back(PO_STORE);
            };
            bool opened = false;
            while (co < ncops) {
                const int op = cops[co++];
                if (op == R_LCACONC) break;
                if (op == R_LCONC) {
                    if (!opened) grp = open_group(ix), opened = true;
                    close_group(true);
                    break;
                }
                if (op == R_CACONC) {
                    const int k = cops[co++];
                    const int o2 = owner_of(k);
                    if (o2 < 0)
                        return fail(c, GBH_ERR_UNSUPPORTED, -1, op, co - 1,
                                    "Ca pool %d is not used by any compartment program", k);
                    if (!need_chips(3)) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "concchip[] too short");
                    NB &nb = nbs[o2];
                    std::vector<int> &PP = nb.n->pool_prog;
                    PP.push_back(PO_CACONC);
                    PP.push_back(nb.pool(k));
                    PP.push_back(chipf(nb, cc));
                    PP.push_back(chipf(nb, cc + 1));
                    PP.push_back(chipf(nb, cc + 2));
                    cc += 3;
                    continue;
                }
                if (op == R_CONC || op == R_FCONC) {
                    if (opened) close_group(op == R_CONC);
                    ix = cops[co++];
                    grp = open_group(ix);
                    opened = true;
                    if (grp < 0)
                        return fail(c, GBH_ERR_UNSUPPORTED, -1, op, co - 1,
                                    "conc %d is not tied to a neuron of a multi-neuron solver", ix);
                    continue;
                }
                if (!opened) {   // ops before the first FCONC act on conc 0
                    grp = open_group(ix);
                    opened = true;
                    if (grp < 0) return fail(c, GBH_ERR_UNSUPPORTED, -1, op, co - 1, "conc 0 has no neuron");
                }
                NB &nb = nbs[grp];
                std::vector<int> &PP = nb.n->pool_prog;
                switch (op) {
                case R_FLUXCONC:
                    if (!need_chips(2)) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "concchip[] too short");
                    PP.insert(PP.end(), {PO_FLUXCONC, chipf(nb, cc), chipf(nb, cc + 1)});
                    cc += 2;
                    break;
                case R_CTAUPUMP:
                    if (!need_chips(2)) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "concchip[] too short");
                    PP.insert(PP.end(), {PO_CTAU, chipf(nb, cc), chipf(nb, cc + 1)});
                    cc += 2;
                    break;
                case R_TAUPUMP: {
                    const int vr = cops[co++];
                    if (!need_chips(5)) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "concchip[] too short");
                    PP.insert(PP.end(), {PO_TAU, vr - nb.n->row0, chipf(nb, cc), chipf(nb, cc + 1), chipf(nb, cc + 2),
                                         chipf(nb, cc + 3), chipf(nb, cc + 4)});
                    cc += 5;
                    break;
                }
                case R_MMPUMP:
                    if (!need_chips(2)) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "concchip[] too short");
                    PP.insert(PP.end(), {PO_MM, chipf(nb, cc), chipf(nb, cc + 1)});
                    cc += 2;
                    break;
                case R_HILLPUMP: {
                    const int h = cops[co++];
                    if (!need_chips(2)) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "concchip[] too short");
                    PP.insert(PP.end(), {PO_HILL, h, chipf(nb, cc), chipf(nb, cc + 1)});
                    cc += 2;
                    break;
                }
                case R_PHILLPUMP: {
                    const int h = cops[co], k = cops[co + 1];
                    co += 2;
                    if (!need_chips(3)) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "concchip[] too short");
                    PP.insert(PP.end(), {PO_PHILL, h, nb.pool(k), chipf(nb, cc), chipf(nb, cc + 1), chipf(nb, cc + 2)});
                    cc += 3;
                    break;
                }
                case R_BUFFER: {
                    const int k = cops[co++];
                    if (!need_chips(3)) return fail(c, GBH_ERR_ARG, -1, op, co - 1, "concchip[] too short");
                    PP.insert(PP.end(), {PO_BUFFER, nb.pool(k), chipf(nb, cc), chipf(nb, cc + 1), chipf(nb, cc + 2)});
                    cc += 3;
                    break;
                }
                case R_POOL:
                    PP.push_back(PO_POOL);
                    break;
                default:
                    return fail(c, GBH_ERR_OPCODE, -1, op, co - 1, "concops opcode %d is not implemented", op);
                }
            }
            // diffusion systems, in the order the reference solves them
            int64_t q0 = d->covals0_start ? d->covals0_start[si] : 0;
            const int64_t q1 = d->covals0_start ? d->covals0_start[si + 1] : 0;
            const int64_t b0 = d->bufvals_start ? d->bufvals_start[si] : 0;
            const int64_t nbufv = d->bufvals_start ? d->bufvals_start[si + 1] - b0 : 0;
            for (int64_t i = ds0; i < ds1; ++i) {
                const int c0 = d->dconc[i], ms = d->nshells[i], w = d->nshrows[i], nfix = d->nshfix[i];
                const int o2 = owner_of(c0);
                if (o2 < 0)
                    return fail(c, GBH_ERR_UNSUPPORTED, -1, 0, i - ds0,
                                "diffusion system %lld is not tied to a neuron", (long long)(i - ds0));
                // covals0 entries it consumes: one per fixed buffer, one or two
                // (inner shells) per diffusible buffer and per shell row
                int64_t nq = 0;
                for (int m = 0; m < ms; ++m) nq += nfix + (int64_t)(w - nfix) * ((m == 0 || m == ms - 1) ? 1 : 2);
                const int nb3 = 3 * (w - 1);
                if (q0 + nq > q1 || (w > 1 && (d->fbufval[i] < 0 || d->fbufval[i] + nb3 > nbufv)))
                    return fail(c, GBH_ERR_ARG, -1, 0, i - ds0, "covals0[]/bufvals[] too short for diffusion system %lld",
                                (long long)(i - ds0));
                NB &nb = nbs[o2];
                Neuron &N = *nb.n;
                N.has_cd = true;
                const int nfac = w > 1 ? ms * w * w : ms + 1, npart = ms * w;
                std::vector<int> &PP = N.pool_prog;
                PP.insert(PP.end(), {PO_DIFF, ms, w, nfix, N.crank, N.nscratch, (int)nq, w > 1 ? nb3 : 0});
                for (int j = 0; j < ms * w; ++j) PP.push_back(nb.pool(c0 + j));
                for (int64_t q = 0; q < nq; ++q) PP.push_back(nb.fld(FS_COV0, q0 + q, d->covals0[q0 + q]));
                if (w > 1)
                    for (int j = 0; j < nb3; ++j) {
                        const int64_t bi = b0 + d->fbufval[i] + j;
                        PP.push_back(nb.fld(FS_BUFV, bi, d->bufvals[bi]));
                    }
                N.nscratch += nfac + npart;
                q0 += nq;
            }
        }
        for (int k = 0; k < ntrees; ++k) {
            nbs[k].n->pool_prog.push_back(0);
            make_key(*nbs[k].n);
        }
    }
    return GBH_OK;
}

}  // namespace

// Solvers are independent, so chunks of them decode on separate threads; the
// chunks are then concatenated in solver order and their synchan constant
// sets merged first-come (the indices a sequential pass would assign; the
// programs and grouping keys of a chunk whose indices move are updated).
// The first error in solver order is the one reported.
namespace {

int decode_chunks(const gbh_batch_desc *d, Decoded &out, gbh_error *err)
{
    Ctx c{d, err, -1};
    if (!d || d->abi_version != GBH_ABI_VERSION)
        return fail(c, GBH_ERR_ARG, -1, 0, -1, "descriptor missing or ABI version mismatch");
    if (d->nsolvers <= 0) return fail(c, GBH_ERR_ARG, -1, 0, -1, "no solvers");
    const int ns = d->nsolvers;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nchunk = std::max(1, std::min({(int)std::min(hw, 32u), ns / 256, ns}));
    struct Chunk {
        int s0 = 0, s1 = 0, rc = GBH_OK;
        std::vector<Neuron> neurons;
        std::vector<double> stab;
        std::vector<int> first;   // neurons before each of its solvers
        gbh_error err{};
    };
    std::vector<Chunk> ch(nchunk);
    // no C++ exception leaves the C ABI: host memory exhaustion is an error code
    auto work = [&](Chunk &k) {
        int si = k.s0;
        try {
            for (; si < k.s1; ++si) {
                k.first.push_back((int)k.neurons.size());
                k.rc = decode_solver(d, si, k.neurons, k.stab, &k.err);
                if (k.rc) return;
            }
        } catch (const std::exception &ex) {
            Ctx ce{d, &k.err, si};
            k.rc = fail(ce, GBH_ERR_ARG, -1, 0, -1, "decoding needs more host memory than is available (%s)",
                        ex.what());
        }
    };
    for (int i = 0; i < nchunk; ++i) {
        ch[i].s0 = (int)((int64_t)ns * i / nchunk);
        ch[i].s1 = (int)((int64_t)ns * (i + 1) / nchunk);
    }
    if (nchunk == 1) {
        work(ch[0]);
    } else {
        std::vector<std::thread> th;
        int started = 0;
        try {
            th.reserve(nchunk);
            for (; started < nchunk; ++started) th.emplace_back(work, std::ref(ch[started]));
        } catch (const std::exception &) {
            // no more threads to be had: the remaining chunks run here
        }
        for (int i = started; i < nchunk; ++i) work(ch[i]);
        for (auto &t : th) t.join();
    }
    out.neurons.clear();
    out.stablist.clear();
    out.solver_first_neuron.assign(ns + 1, 0);
    size_t total = 0;
    for (const Chunk &k : ch) {
        if (k.rc) {
            if (err) *err = k.err;
            return k.rc;
        }
        total += k.neurons.size();
    }
    out.neurons.reserve(total);
    for (Chunk &k : ch) {
        std::vector<int> remap(k.stab.size() / 4);
        bool moved = false;
        for (size_t q = 0; q + 4 <= k.stab.size(); q += 4) {
            int g = -1;
            for (size_t r = 0; r + 4 <= out.stablist.size(); r += 4)
                if (memcmp(&out.stablist[r], &k.stab[q], 4 * sizeof(double)) == 0) { g = (int)r; break; }
            if (g < 0) {
                g = (int)out.stablist.size();
                out.stablist.insert(out.stablist.end(), k.stab.begin() + q, k.stab.begin() + q + 4);
            }
            remap[q / 4] = g;
            moved = moved || g != (int)q;
        }
        const int base = (int)out.neurons.size();
        for (int si = k.s0; si < k.s1; ++si) out.solver_first_neuron[si] = base + k.first[si - k.s0];
        for (Neuron &N : k.neurons) {
            if (moved && !N.stab_pos.empty()) {
                for (int p : N.stab_pos) N.prog[p] = remap[N.prog[p] / 4];
                make_key(N);
            }
            out.neurons.push_back(std::move(N));
        }
        std::vector<Neuron>().swap(k.neurons);
    }
    out.solver_first_neuron[ns] = (int)out.neurons.size();
    return GBH_OK;
}

}  // namespace

int decode_batch(const gbh_batch_desc *d, Decoded &out, gbh_error *err)
{
    try {
        return decode_chunks(d, out, err);
    } catch (const std::exception &ex) {
        Ctx c{d, err, -1};
        out.neurons.clear();
        return fail(c, GBH_ERR_ARG, -1, 0, -1, "decoding needs more host memory than is available (%s)", ex.what());
    }
}

}  // namespace gbh
