// gbh_hsolve.cpp -- the hsolve-level ABI (include/gbh_hsolve.h): every
// registered hsolve joins one batch engine, stepped once per simulation step
// by the first solver the scheduler calls in that step.
//
// The reference keeps one accelerator state per hsolve in a process-wide
// list and, when no solver has a spike detector, lets the first call of a
// step dispatch every solver (genesis/src/hines/cuda/cuda_hsolve.c:64-145).
// Here the batch is one engine over all solvers' arrays, spike detectors
// included: their synapses onto solvers of the batch become device synapses
// (gbh_synapses), so a step needs no GENESIS messaging between solvers.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "gbh_hsolve.h"

namespace {

struct Registry {
    std::vector<gbh_hs_solver> sv;
    gbh_engine *e = nullptr;
    bool dirty = false;
    bool stepped = false;
    long long stamp = 0;
    long long synced_stamp = -1;    // stamp of the flat state images below
    // flat images in the batch layout
    std::vector<int64_t> ops_s, chip_s, funcs_s, rav_s, vm_s, giv_s, stab_s, conc_s, cops_s, cchip_s, itot_s;
    std::vector<int> ops, funcs, cops;
    std::vector<double> chip, rav, vm, giv, stab, conc, cchip, itot;
    std::vector<double> in_vals;
    std::vector<int64_t> spikes_last;
    bool any_out = false, any_spike_host = false, any_itot = false;
    std::string err;
};

Registry &reg()
{
    static Registry r;
    return r;
}

template <typename T>
void cat(std::vector<int64_t> &start, std::vector<T> &flat, size_t i, const T *p, int64_t n)
{
    if (start.empty()) start.push_back(0);
    if (n > 0 && p) flat.insert(flat.end(), p, p + n);
    else if (n > 0) flat.insert(flat.end(), (size_t)n, T());
    start.push_back((int64_t)flat.size());
    (void)i;
}

// Entries of a table set's arrays the engine reads: xdivs + 1 rows of
// tablist and xvals, ydivs + 1 of yvals.
int64_t tab_len(const gbh_tables &t) { return t.ncols ? (int64_t)(t.xdivs + 1) * t.ncols : 0; }
int64_t xv_len(const gbh_tables &t) { return t.ncols ? t.xdivs + 1 : 0; }
int64_t yv_len(const gbh_tables &t) { return t.ydivs > 0 ? t.ydivs + 1 : 0; }

uint64_t mix(uint64_t h, const void *p, size_t n)
{
    const unsigned char *b = (const unsigned char *)p;
    for (size_t k = 0; k < n; ++k) h = (h ^ b[k]) * 1099511628211ULL;   // FNV-1a
    return h;
}

uint64_t table_hash(const gbh_tables &t)
{
    uint64_t h = 1469598103934665603ULL;
    const double sc[4] = {t.xmin, t.invdx, t.ymin, t.invdy};
    const int ic[3] = {t.ncols, t.xdivs, t.ydivs};
    h = mix(h, sc, sizeof(sc));
    h = mix(h, ic, sizeof(ic));
    if (t.tablist) h = mix(h, t.tablist, sizeof(double) * tab_len(t));
    if (t.xvals) h = mix(h, t.xvals, sizeof(double) * xv_len(t));
    if (t.yvals) h = mix(h, t.yvals, sizeof(double) * yv_len(t));
    return h;
}

bool same_arr(const double *a, const double *b, int64_t n)
{
    if (a == b || n == 0) return true;
    if (!a || !b) return false;
    return memcmp(a, b, sizeof(double) * n) == 0;
}

bool same_tables(const gbh_tables &a, const gbh_tables &b)
{
    return a.ncols == b.ncols && a.xdivs == b.xdivs && a.ydivs == b.ydivs && a.xmin == b.xmin &&
           a.invdx == b.invdx && a.ymin == b.ymin && a.invdy == b.invdy &&
           same_arr(a.tablist, b.tablist, tab_len(a)) && same_arr(a.xvals, b.xvals, xv_len(a)) &&
           same_arr(a.yvals, b.yvals, yv_len(a));
}

int fail(const char *msg)
{
    reg().err = msg;
    fprintf(stderr, "gbh_hsolve: %s\n", msg);
    return GBH_ERR_ARG;
}

// Copies the batch state from the engine into the solvers' own arrays.
void scatter_all(Registry &r)
{
    for (size_t i = 0; i < r.sv.size(); ++i) {
        gbh_hs_solver &s = r.sv[i];
        if (s.vm) memcpy(s.vm, &r.vm[r.vm_s[i]], sizeof(double) * s.ncompts);
        if (s.chip) memcpy(s.chip, &r.chip[r.chip_s[i]], sizeof(double) * s.nchips);
        if (s.conc && s.nconcs) memcpy(s.conc, &r.conc[r.conc_s[i]], sizeof(double) * s.nconcs);
        if (s.ops) memcpy(s.ops, &r.ops[r.ops_s[i]], sizeof(int) * s.nops);
    }
}

int pull_state(Registry &r)
{
    if (r.synced_stamp == r.stamp && r.stepped) return GBH_OK;
    const int rc = gbh_get_state(r.e, r.vm.data(), r.chip.data(), r.conc.data(), r.ops.data());
    if (rc) return rc;
    if (r.any_itot && gbh_get_itotal(r.e, r.itot.data())) return GBH_ERR_CUDA;
    r.synced_stamp = r.stamp;
    return GBH_OK;
}

int build(Registry &r)
{
    if (r.e) {   // carry the running state over into the solvers' arrays first
        r.synced_stamp = -1;
        if (pull_state(r) == GBH_OK) scatter_all(r);
        gbh_destroy(r.e);
        r.e = nullptr;
    }
    const size_t n = r.sv.size();
    if (!n) return fail("no solver registered");
    for (auto *v : {&r.ops_s, &r.chip_s, &r.funcs_s, &r.rav_s, &r.vm_s, &r.giv_s, &r.stab_s, &r.conc_s, &r.cops_s,
                    &r.cchip_s, &r.itot_s})
        v->clear();
    r.ops.clear(); r.funcs.clear(); r.cops.clear();
    r.chip.clear(); r.rav.clear(); r.vm.clear(); r.giv.clear(); r.stab.clear(); r.conc.clear(); r.cchip.clear();
    r.itot.clear();
    std::vector<int> method(n), chanmode(n), calcmode(n), tset(n), storemode(n);
    std::vector<gbh_tables> tabs;
    std::multimap<uint64_t, int> tab_of;
    // difshell systems
    std::vector<int64_t> diff_s(1, 0), cov_s(1, 0), buf_s(1, 0);
    std::vector<int> dconc, nsh, nrow, nfix, fbuf;
    std::vector<double> cov, buf;
    bool any_diff = false;
    r.any_out = r.any_spike_host = r.any_itot = false;
    const double dt = r.sv[0].dt;
    for (size_t i = 0; i < n; ++i) {
        const gbh_hs_solver &s = r.sv[i];
        if (s.dt != dt) return fail("all solvers of a batch step with one dt");
        method[i] = s.method == 11 ? 11 : 10;   // CRANK_INT, else BEULER
        chanmode[i] = s.chanmode;
        calcmode[i] = s.calcmode;
        storemode[i] = s.storemode;
        // one table set per distinct table: every hsolve builds its own copy
        // (duplicate_tables, hines_chip_init.c:1262-1400), identical across the
        // solvers of one cell type
        const uint64_t hk = table_hash(s.tables);
        int found = -1;
        for (auto it = tab_of.lower_bound(hk); it != tab_of.end() && it->first == hk && found < 0; ++it)
            if (same_tables(tabs[it->second], s.tables)) found = it->second;
        if (found < 0) {
            found = (int)tabs.size();
            tab_of.emplace(hk, found);
            tabs.push_back(s.tables);
        }
        tset[i] = found;
        cat(r.ops_s, r.ops, i, s.ops, s.nops);
        cat(r.chip_s, r.chip, i, s.chip, s.nchips);
        cat(r.funcs_s, r.funcs, i, s.funcs, s.nfuncs);
        cat(r.rav_s, r.rav, i, s.ravals, s.nravals);
        cat(r.vm_s, r.vm, i, (const double *)s.vm, s.ncompts);
        cat(r.giv_s, r.giv, i, (const double *)s.givals, s.ngivals);
        cat(r.stab_s, r.stab, i, s.stablist, s.nstab);
        cat(r.conc_s, r.conc, i, (const double *)s.conc, s.nconcs);
        cat(r.cops_s, r.cops, i, s.concops, s.nconcops);
        cat(r.cchip_s, r.cchip, i, s.concchip, s.nconcchips);
        cat(r.itot_s, r.itot, i, (const double *)nullptr, s.storemode ? s.nelm_names : 0);
        r.any_itot = r.any_itot || (s.storemode && s.nelm_names > 0);
        for (int k = 0; k < s.ndiffs; ++k) {
            dconc.push_back(s.dconc[k]);
            nsh.push_back(s.nshells[k]);
            nrow.push_back(s.nshrows[k]);
            nfix.push_back(s.nshfix[k]);
            fbuf.push_back(s.fbufval[k]);
        }
        if (s.ndiffs) any_diff = true;
        diff_s.push_back((int64_t)dconc.size());
        if (s.ncovals0) cov.insert(cov.end(), s.covals0, s.covals0 + s.ncovals0);
        cov_s.push_back((int64_t)cov.size());
        if (s.nbufvals) buf.insert(buf.end(), s.bufvals, s.bufvals + s.nbufvals);
        buf_s.push_back((int64_t)buf.size());
        r.any_out = r.any_out || s.has_outputs;
        r.any_spike_host = r.any_spike_host || s.on_spike;
    }
    if (r.itot.empty()) r.itot.push_back(0.0);
    gbh_batch_desc d;
    memset(&d, 0, sizeof(d));
    d.abi_version = GBH_ABI_VERSION;
    d.nsolvers = (int)n;
    d.dt = dt;
    d.method = method.data();
    d.chanmode = chanmode.data();
    d.calcmode = calcmode.data();
    d.table_set = tset.data();
    d.ntables = (int)tabs.size();
    d.tables = tabs.data();
    d.ops_start = r.ops_s.data(); d.ops = r.ops.data();
    d.chip_start = r.chip_s.data(); d.chip = r.chip.data();
    d.funcs_start = r.funcs_s.data(); d.funcs = r.funcs.data();
    d.ravals_start = r.rav_s.data(); d.ravals = r.rav.data();
    d.vm_start = r.vm_s.data(); d.vm = r.vm.data();
    d.givals_start = r.giv_s.data(); d.givals = r.giv.data();
    d.stab_start = r.stab_s.data(); d.stablist = r.stab.data();
    d.conc_start = r.conc_s.data(); d.conc = r.conc.data();
    d.concops_start = r.cops_s.data(); d.concops = r.cops.data();
    d.concchip_start = r.cchip_s.data(); d.concchip = r.cchip.data();
    if (any_diff) {
        d.diff_start = diff_s.data();
        d.dconc = dconc.data();
        d.nshells = nsh.data();
        d.nshrows = nrow.data();
        d.nshfix = nfix.data();
        d.fbufval = fbuf.data();
        d.covals0_start = cov_s.data();
        d.covals0 = cov.data();
        d.bufvals_start = buf_s.data();
        d.bufvals = buf.data();
    }
    if (r.any_itot) {
        d.storemode = storemode.data();
        d.itotal_start = r.itot_s.data();
    }
    // synapses: CSR over the source solvers
    std::vector<int64_t> src_start(1, 0);
    std::vector<int> tsolver, top, tdelay;
    std::vector<double> tweight;
    for (size_t i = 0; i < n; ++i) {
        const gbh_hs_solver &s = r.sv[i];
        for (int k = 0; k < s.nsynapses; ++k) {
            const gbh_hs_synapse &y = s.synapses[k];
            if (y.target < 0 || y.target >= (int)n) return fail("synapse onto a solver outside the batch");
            tsolver.push_back(y.target);
            top.push_back(y.target_op);
            tweight.push_back(y.weight);
            tdelay.push_back(y.delay_steps);
        }
        src_start.push_back((int64_t)tsolver.size());
    }
    gbh_synapses syn;
    memset(&syn, 0, sizeof(syn));
    syn.nsynapses = (int64_t)tsolver.size();
    syn.src_start = src_start.data();
    syn.target_solver = tsolver.data();
    syn.target_op = top.data();
    syn.weight = tweight.data();
    syn.delay_steps = tdelay.data();
    gbh_options opt;
    memset(&opt, 0, sizeof(opt));
    gbh_error err;
    r.e = gbh_create(&d, syn.nsynapses ? &syn : nullptr, &opt, &err);
    if (!r.e) {
        char msg[400];
        snprintf(msg, sizeof(msg), "batch setup failed: solver %d row %d opcode %d: %s", err.solver, err.row,
                 err.opcode, err.message);
        reg().err = msg;
        fprintf(stderr, "gbh_hsolve: %s\n", msg);
        return err.code ? err.code : GBH_ERR_ARG;
    }
    // h_in_msgs inputs of every solver, in solver then list order
    std::vector<int> isol, ikind;
    std::vector<int64_t> iidx;
    std::vector<double> isa, isb;
    for (size_t i = 0; i < n; ++i)
        for (int k = 0; k < r.sv[i].ninputs; ++k) {
            const gbh_hs_input &in = r.sv[i].inputs[k];
            isol.push_back((int)i);
            ikind.push_back(in.kind);
            iidx.push_back(in.index);
            isa.push_back(in.sa);
            isb.push_back(in.sb);
        }
    r.in_vals.assign(isol.size(), 0.0);
    if (!isol.empty() && gbh_register_inputs_typed(r.e, (int)isol.size(), isol.data(), ikind.data(), iidx.data(),
                                                   isa.data(), isb.data()) != GBH_OK)
        return fail(gbh_last_error());
    r.spikes_last.assign(n, 0);
    if (r.any_spike_host) gbh_get_spike_counts(r.e, r.spikes_last.data());
    r.dirty = false;
    r.synced_stamp = -1;
    return GBH_OK;
}

}  // namespace

extern "C" {

int gbh_hs_register(const gbh_hs_solver *s)
{
    if (!s || s->ncompts <= 0 || !s->ops || !s->chip || !s->funcs || !s->vm) return fail("incomplete solver");
    Registry &r = reg();
    r.sv.push_back(*s);
    r.dirty = true;
    return (int)r.sv.size() - 1;
}

int gbh_hs_set_synapses(int id, int nsynapses, const gbh_hs_synapse *synapses, void (*on_spike)(void *ctx),
                        void *spike_ctx)
{
    Registry &r = reg();
    if (id < 0 || id >= (int)r.sv.size() || nsynapses < 0 || (nsynapses && !synapses)) return GBH_ERR_ARG;
    gbh_hs_solver &s = r.sv[id];
    s.nsynapses = nsynapses;
    s.synapses = synapses;
    s.on_spike = on_spike;
    s.spike_ctx = spike_ctx;
    r.dirty = true;
    return GBH_OK;
}

int gbh_hs_step(int id, long long stamp)
{
    Registry &r = reg();
    if (id < 0 || id >= (int)r.sv.size()) return GBH_ERR_ARG;
    if (r.stepped && stamp == r.stamp) return 1;   // this step is done for every solver
    if (r.dirty || !r.e) {
        const int rc = build(r);
        if (rc) return rc;
    }
    // the first call of the step: every solver's inputs, one step of the batch
    size_t q = 0;
    for (const gbh_hs_solver &s : r.sv)
        for (int k = 0; k < s.ninputs; ++k) r.in_vals[q++] = s.inputs[k].value(s.inputs[k].ctx);
    if (q && gbh_set_inputs_async(r.e, r.in_vals.data(), nullptr) != GBH_OK) return GBH_ERR_CUDA;
    int rc = gbh_run(r.e, 1);
    if (rc) {
        reg().err = gbh_last_error();
        return rc;
    }
    r.stamp = stamp;
    r.stepped = true;
    if (r.any_out) {   // h_out_msgs reads vm (and itotal) of these solvers
        if ((rc = gbh_get_state(r.e, r.vm.data(), nullptr, nullptr, nullptr)) != GBH_OK) return rc;
        if (r.any_itot && (rc = gbh_get_itotal(r.e, r.itot.data())) != GBH_OK) return rc;
        for (size_t i = 0; i < r.sv.size(); ++i) {
            gbh_hs_solver &s = r.sv[i];
            if (!s.has_outputs) continue;
            memcpy(s.vm, &r.vm[r.vm_s[i]], sizeof(double) * s.ncompts);
            if (s.storemode && s.itotal && s.nelm_names)
                memcpy(s.itotal, &r.itot[r.itot_s[i]], sizeof(double) * s.nelm_names);
        }
    }
    if (r.any_spike_host) {   // spikes for targets outside the batch
        std::vector<int64_t> now(r.sv.size(), 0);
        if ((rc = gbh_get_spike_counts(r.e, now.data())) != GBH_OK) return rc;
        for (size_t i = 0; i < r.sv.size(); ++i) {
            for (int64_t k = r.spikes_last[i]; k < now[i]; ++k)
                if (r.sv[i].on_spike) r.sv[i].on_spike(r.sv[i].spike_ctx);
            r.spikes_last[i] = now[i];
        }
    }
    return 1;
}

int gbh_hs_sync(int id)
{
    Registry &r = reg();
    if (id < 0 || id >= (int)r.sv.size()) return GBH_ERR_ARG;
    if (!r.e) return GBH_OK;   // nothing stepped yet: the host arrays are current
    const int rc = pull_state(r);
    if (rc) return rc;
    gbh_hs_solver &s = r.sv[id];
    memcpy(s.vm, &r.vm[r.vm_s[id]], sizeof(double) * s.ncompts);
    memcpy(s.chip, &r.chip[r.chip_s[id]], sizeof(double) * s.nchips);
    if (s.conc && s.nconcs) memcpy(s.conc, &r.conc[r.conc_s[id]], sizeof(double) * s.nconcs);
    memcpy(s.ops, &r.ops[r.ops_s[id]], sizeof(int) * s.nops);
    if (s.storemode && s.itotal && s.nelm_names)
        memcpy(s.itotal, &r.itot[r.itot_s[id]], sizeof(double) * s.nelm_names);
    return GBH_OK;
}

int gbh_hs_push(int id)
{
    Registry &r = reg();
    if (id < 0 || id >= (int)r.sv.size()) return GBH_ERR_ARG;
    if (!r.e || r.dirty) return GBH_OK;   // the next build copies the host arrays
    r.synced_stamp = -1;
    int rc = pull_state(r);
    if (rc) return rc;
    const gbh_hs_solver &s = r.sv[id];
    memcpy(&r.vm[r.vm_s[id]], s.vm, sizeof(double) * s.ncompts);
    memcpy(&r.chip[r.chip_s[id]], s.chip, sizeof(double) * s.nchips);
    if (s.conc && s.nconcs) memcpy(&r.conc[r.conc_s[id]], s.conc, sizeof(double) * s.nconcs);
    rc = gbh_set_state(r.e, r.vm.data(), r.chip.data(), r.conc.empty() ? nullptr : r.conc.data());
    r.synced_stamp = -1;
    return rc;
}

int gbh_hs_stats(gbh_stats *st)
{
    Registry &r = reg();
    if (!st || !r.e) return GBH_ERR_ARG;
    return gbh_get_stats(r.e, st);
}

int gbh_hs_count(void) { return (int)reg().sv.size(); }

void gbh_hs_cleanup(void)
{
    Registry &r = reg();
    if (r.e) gbh_destroy(r.e);
    r = Registry();
}

}  // extern "C"
