/*
 * ref_setup.c -- runs the reference's own SETUP code for the elimination
 * program on a compartment tree given as flat arrays.
 *
 * TEST INFRASTRUCTURE ONLY. Compiled together with the reference source
 * genesis/src/hines/hines_init.c (never copied into this repository) into
 * oracle/_ref/libhsetup_ref.so by oracle/Makefile. tests/golden/make_symcompt.py
 * calls it to produce golden funcs[]/ravals[] vectors, above all for
 * symmetric compartments, whose elimination program (COPY_ARRAY,
 * FASTSIBARRAY_ELIM, SIBARRAY_ELIM tokens) only the reference's setup emits.
 *
 * The steps follow h_init (hines_init.c:246-296: kids filled in element order,
 * do_hnum over every root, kids bubble-sorted by Hines number) and the two
 * passes of h_funcs_init (hines_init.c:361-1273: count, then fill) with
 * chanmode 0 so the diagonal terms land in hsolve->diagonals.
 */
#include <stdlib.h>
#include <string.h>
#include "hines_ext.h"

extern int do_hnum();
extern int h_funcs_init();

/* symbols hines_init.c references from the rest of GENESIS; only h_init
 * and its helpers (not called here) use them */
void Error(void) {}
void ErrorMessage(void) {}
void HsolveBlock(void) {}
char *Pathname(void) { return "ref_setup"; }
void SetWorkingElement(void) {}
Element *WorkingElement(void) { return NULL; }
ElementList *WildcardGetElement(void) { return NULL; }
int Strindex(void) { return -1; }

static GenesisObject ref_object;
GenesisObject *BaseObject(Element *e)
{
    (void)e;
    return &ref_object;
}

/*
 * n compartments; parent[c] is the parent element of compartment c (-1 for a
 * root), Ra/Cm/Rm its float fields; method 10 (backward Euler) or 11
 * (Crank-Nicolson). Outputs: hnum[n] (element -> row), funcs[*nfuncs],
 * ravals[*nravals], diag[n] (the constant diagonal term of each row).
 * Returns 0, -1 when a buffer is too small (its needed size is still written
 * to *nfuncs / *nravals) or -2 when the reference's setup reports an error.
 */
int ref_funcs_init(int n, const int *parent, const float *Ra, const float *Cm, const float *Rm,
                   int method, double dt, int symflag, int *hnum_out, int *elmnum_out,
                   int *funcs, int *nfuncs, double *ravals, int *nravals, double *diag)
{
    Hsolve h;
    struct compartment_type *cs = calloc((size_t)n, sizeof(*cs));
    Element **compts = calloc((size_t)n, sizeof(*compts));
    int *nkids = calloc((size_t)n, sizeof(int));
    int **kids = calloc((size_t)n, sizeof(int *));
    int *fill = calloc((size_t)n, sizeof(int));
    int *hnum = calloc((size_t)n, sizeof(int));
    int *elmnum = calloc((size_t)n, sizeof(int));
    int *par = calloc((size_t)n, sizeof(int));
    double *diagonals = calloc((size_t)n, sizeof(double));
    int i, j, k, f, cnt, rc = 0, nf, nr;

    memset(&h, 0, sizeof(h));
    for (i = 0; i < n; i++) {
        cs[i].Ra = Ra[i];
        cs[i].Cm = Cm[i];
        cs[i].Rm = Rm[i];
        compts[i] = (Element *)&cs[i];
        par[i] = parent[i];
        if (parent[i] >= 0) nkids[parent[i]]++;
    }
    for (i = 0; i < n; i++) kids[i] = nkids[i] ? calloc((size_t)nkids[i], sizeof(int)) : NULL;
    for (j = 0; j < n; j++)
        if (par[j] != -1) kids[par[j]][fill[par[j]]++] = j;
    h.name = "ref_setup";
    h.ncompts = n;
    h.symflag = symflag;
    h.compts = compts;
    h.parents = par;
    h.nkids = nkids;
    h.kids = kids;
    h.hnum = hnum;
    h.elmnum = elmnum;
    h.diagonals = diagonals;
    h.chanmode = 0;
    h.dt = dt;
    ref_object.method = method;

    cnt = n - 1;
    for (i = 0; i < n; i++)
        if (par[i] == -1) do_hnum(&h, i, &cnt, elmnum);
    for (i = 0; i < n; i++) {
        j = elmnum[i];
        f = 1;
        while (f) {
            f = 0;
            for (k = 1; k < nkids[j]; k++) {
                if (hnum[kids[j][k - 1]] > hnum[kids[j][k]]) {
                    int t = kids[j][k - 1];
                    kids[j][k - 1] = kids[j][k];
                    kids[j][k] = t;
                    f = 1;
                }
            }
        }
    }

    h.nfuncs = 0;
    if (h_funcs_init(&h) != 0) { rc = -2; goto done; }   /* counting pass */
    nf = h.nfuncs;
    nr = h.nravals;
    if (nf > *nfuncs || nr > *nravals) {
        *nfuncs = nf;
        *nravals = nr;
        rc = -1;
        goto done;
    }
    if (h_funcs_init(&h) != 0) { rc = -2; goto done; }   /* filling pass */
    *nfuncs = nf;
    *nravals = nr;
    memcpy(funcs, h.funcs, (size_t)nf * sizeof(int));
    if (nr) memcpy(ravals, h.ravals, (size_t)nr * sizeof(double));
    memcpy(diag, diagonals, (size_t)n * sizeof(double));
    memcpy(hnum_out, hnum, (size_t)n * sizeof(int));
    memcpy(elmnum_out, elmnum, (size_t)n * sizeof(int));

done:
    free(h.funcs);
    free(h.ravals);
    if (h.ravptr) {
        for (i = 0; i < n; i++) free(h.ravptr[i]);
        free(h.ravptr);
    }
    free(h.fwd_seg_start);
    free(h.bwd_seg_start);
    free(h.fwd_root_row);
    free(h.fwd_raval_start);
    free(h.bwd_raval_start);
    for (i = 0; i < n; i++) free(kids[i]);
    free(cs); free(compts); free(nkids); free(kids); free(fill); free(hnum); free(elmnum); free(par);
    free(diagonals);
    return rc;
}
