/*
 * ORACLE -- test infrastructure only.
 *
 * Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
 * load this code, and only as the checker (or as the timed CPU stand-in for
 * the reference).  The shipped library never links or calls it.
 *
 * What it is: a CPU restatement of the reference solver's two-watched-literal
 * BCP applied to a partial trail, in the reference's own processing order, so
 * that the implied literals (in order), their reason clauses, the conflict
 * flag and the conflicting clause are identical to what the reference computes.
 * Data structures are this file's own (flat arrays, an arena for list growth);
 * only the observable order is kept.
 *
 * Reference behaviour restated (paths inside the reference project, src/):
 *  - literal = 2*var + sign, sign 1 = positive       SATSolver/SolverTypes.cu:6-42
 *  - initial watches: the two literals whose var lists are shortest at
 *    insertion time (strict '<', so ties keep the earlier literal), then
 *    add_first to var(lit_a) and var(lit_b)
 *        BCPStrategy/ClauseListStructure.cu:101-148, WatchedClausesList.cu:356-364
 *    -> every per-var list starts in decreasing clause order.
 *  - trail application: every trail literal is assigned first
 *        SATSolver/VariablesStateHandler.cu:35-59
 *    then new_decision() per literal in trail order with one shared pending
 *    list, stopping at the first conflict
 *        ConflictAnalysis/ConflictAnalyzerWithWatchedLits.cu:56-73
 *  - new_decision: snapshot the var's list, process each entry, then recurse
 *    depth-first on the implications found by this call, in order
 *        BCPStrategy/WatchedClausesList.cu:46-101
 *  - process_clause          WatchedClausesList.cu:103-221
 *  - is_currently_consistent WatchedClausesList.cu:223-241 (assignment or
 *    pending list; both live in val[] here)
 *  - handle_implication      WatchedClausesList.cu:253-282 (push only when the
 *    literal is unassigned; the clause is blocked either way)
 *  - block_clause            ClauseListStructure.cu:150-164
 *  - switch_watched_literal  ClauseListStructure.cu:73-92 (remove from the old
 *    var's list, add_first to the new var's list)
 *
 * List representation: a clause never returns to a var whose literal it
 * stopped watching (watches only leave inconsistent literals and nothing is
 * unassigned inside one BCP call; clauses have distinct vars).  So the current
 * list of var v is: clauses add_first'ed to v (newest first) followed by the
 * initial list of v, keeping only entries whose clause still watches v and is
 * not blocked.  That is exactly the reference's linked list.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define ORC_OK 0
#define ORC_ERR_ARG (-1)
#define ORC_ERR_FORMULA (-2)
#define ORC_ERR_NOMEM (-3)

/* per-trail status codes */
#define ORC_BCP_NO_CONFLICT 0
#define ORC_BCP_CONFLICT 1
#define ORC_BCP_OVERFLOW (-1)
#define ORC_BCP_BAD_TRAIL (-2)

typedef struct {
    int32_t n_vars;
    int64_t n_clauses;
    int32_t *lits;   /* internal encoding */
    int64_t *coff;   /* n_clauses + 1 */
    int32_t *iw1, *iw2;       /* initial watch indices */
    int64_t *w0off;           /* n_vars + 1 */
    int32_t *w0cl;            /* initial per-var lists, head first */
} orc_bcp;

static inline int32_t lit_of_dimacs(int32_t d) { return d > 0 ? 2 * (d - 1) + 1 : 2 * (-d - 1); }
static inline int32_t dimacs_of_lit(int32_t l) { return (l & 1) ? (l >> 1) + 1 : -((l >> 1) + 1); }

void orc_bcp_destroy(orc_bcp *f)
{
    if (!f) return;
    free(f->lits); free(f->coff); free(f->iw1); free(f->iw2);
    free(f->w0off); free(f->w0cl); free(f);
}

/* Builds the internal formula and the reference's initial watches.
 * Clauses must be clean: length >= 2 and distinct variables (what the
 * reference's preprocessing leaves, Preprocessing/RepeatedLiteralsRemover.cu). */
orc_bcp *orc_bcp_create(const int32_t *dimacs, const int64_t *coff, int32_t n_vars, int64_t n_clauses)
{
    if (n_vars <= 0 || n_clauses < 0) return NULL;
    orc_bcp *f = (orc_bcp *)calloc(1, sizeof(orc_bcp));
    int64_t nl = coff[n_clauses];
    f->n_vars = n_vars; f->n_clauses = n_clauses;
    f->lits = (int32_t *)malloc(sizeof(int32_t) * (nl ? nl : 1));
    f->coff = (int64_t *)malloc(sizeof(int64_t) * (n_clauses + 1));
    f->iw1 = (int32_t *)malloc(sizeof(int32_t) * (n_clauses ? n_clauses : 1));
    f->iw2 = (int32_t *)malloc(sizeof(int32_t) * (n_clauses ? n_clauses : 1));
    f->w0off = (int64_t *)calloc(n_vars + 1, sizeof(int64_t));
    f->w0cl = (int32_t *)malloc(sizeof(int32_t) * (2 * n_clauses + 1));
    int64_t *size = (int64_t *)calloc(n_vars, sizeof(int64_t));
    if (!f->lits || !f->coff || !f->iw1 || !f->iw2 || !f->w0off || !f->w0cl || !size) {
        free(size); orc_bcp_destroy(f); return NULL;
    }
    memcpy(f->coff, coff, sizeof(int64_t) * (n_clauses + 1));
    for (int64_t i = 0; i < nl; i++) {
        int32_t d = dimacs[i];
        if (d == 0 || d > n_vars || d < -n_vars) { free(size); orc_bcp_destroy(f); return NULL; }
        f->lits[i] = lit_of_dimacs(d);
    }
    /* sequential initial-watch choice: list sizes grow as clauses are added */
    for (int64_t c = 0; c < n_clauses; c++) {
        int64_t b = coff[c], k = coff[c + 1] - coff[c];
        if (k < 2) { free(size); orc_bcp_destroy(f); return NULL; }
        int64_t sv = INT64_MAX - 1, sv2 = INT64_MAX;
        int32_t s1 = -1, s2 = -1;
        for (int64_t i = 0; i < k; i++) {
            int64_t cur = size[f->lits[b + i] >> 1];
            if (cur < sv) { s2 = s1; sv2 = sv; sv = cur; s1 = (int32_t)i; }
            else if (cur < sv2) { sv2 = cur; s2 = (int32_t)i; }
        }
        int32_t v1 = f->lits[b + s1] >> 1, v2 = f->lits[b + s2] >> 1;
        if (v1 == v2) { free(size); orc_bcp_destroy(f); return NULL; }
        f->iw1[c] = s1; f->iw2[c] = s2;
        size[v1]++; size[v2]++;
    }
    for (int32_t v = 0; v < n_vars; v++) f->w0off[v + 1] = f->w0off[v] + size[v];
    /* add_first => list order is decreasing clause index */
    int64_t *fill = size; /* reuse as cursor */
    for (int32_t v = 0; v < n_vars; v++) fill[v] = f->w0off[v];
    for (int64_t c = n_clauses - 1; c >= 0; c--) {
        int32_t v1 = f->lits[coff[c] + f->iw1[c]] >> 1, v2 = f->lits[coff[c] + f->iw2[c]] >> 1;
        f->w0cl[fill[v1]++] = (int32_t)c;
        f->w0cl[fill[v2]++] = (int32_t)c;
    }
    free(size);
    return f;
}

int orc_bcp_initial_watches(const orc_bcp *f, int32_t *w1, int32_t *w2)
{
    memcpy(w1, f->iw1, sizeof(int32_t) * f->n_clauses);
    memcpy(w2, f->iw2, sizeof(int32_t) * f->n_clauses);
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* per-worker scratch, reset through touched lists                     */
typedef struct {
    int8_t *val;       /* 0 undef, 1 true, 2 false (trail + pending) */
    int32_t *cw1, *cw2;
    uint8_t *blk, *touched;
    int32_t *tclauses; int64_t ntc, captc;
    int32_t *dhead;    /* -1 = empty */
    int32_t *dvars; int64_t ndv, capdv;
    int32_t *ar_cl, *ar_next; int64_t nar, capar;
    int32_t *snap; int64_t capsnap;
    int64_t *fr_j, *fr_e; int64_t capfr;
} orc_ws;

static int grow32(int32_t **p, int64_t *cap, int64_t need)
{
    if (need <= *cap) return 0;
    int64_t nc = *cap ? *cap : 1024;
    while (nc < need) nc *= 2;
    int32_t *q = (int32_t *)realloc(*p, sizeof(int32_t) * nc);
    if (!q) return -1;
    *p = q; *cap = nc; return 0;
}

static int ws_init(orc_ws *w, const orc_bcp *f)
{
    memset(w, 0, sizeof(*w));
    w->val = (int8_t *)calloc(f->n_vars, 1);
    w->cw1 = (int32_t *)malloc(sizeof(int32_t) * (f->n_clauses + 1));
    w->cw2 = (int32_t *)malloc(sizeof(int32_t) * (f->n_clauses + 1));
    w->blk = (uint8_t *)calloc(f->n_clauses + 1, 1);
    w->touched = (uint8_t *)calloc(f->n_clauses + 1, 1);
    w->dhead = (int32_t *)malloc(sizeof(int32_t) * f->n_vars);
    if (!w->val || !w->cw1 || !w->cw2 || !w->blk || !w->touched || !w->dhead) return -1;
    memcpy(w->cw1, f->iw1, sizeof(int32_t) * f->n_clauses);
    memcpy(w->cw2, f->iw2, sizeof(int32_t) * f->n_clauses);
    for (int32_t v = 0; v < f->n_vars; v++) w->dhead[v] = -1;
    return 0;
}

static void ws_free(orc_ws *w)
{
    free(w->val); free(w->cw1); free(w->cw2); free(w->blk); free(w->touched);
    free(w->tclauses); free(w->dhead); free(w->dvars); free(w->ar_cl); free(w->ar_next);
    free(w->snap); free(w->fr_j); free(w->fr_e);
}

static inline int cons(const orc_ws *w, int32_t l)
{
    int8_t a = w->val[l >> 1];
    return a == 0 || a == ((l & 1) ? 1 : 2);
}

static int touch(orc_ws *w, int32_t c)
{
    if (w->touched[c]) return 0;
    if (grow32(&w->tclauses, &w->captc, w->ntc + 1)) return -1;
    w->touched[c] = 1; w->tclauses[w->ntc++] = c;
    return 0;
}

static int add_first(orc_ws *w, int32_t v, int32_t c)
{
    int64_t capn = w->capar;
    if (grow32(&w->ar_cl, &w->capar, w->nar + 1)) return -1;
    if (capn != w->capar) {
        int32_t *q = (int32_t *)realloc(w->ar_next, sizeof(int32_t) * w->capar);
        if (!q) return -1;
        w->ar_next = q;
    }
    if (w->dhead[v] == -1) {
        if (grow32(&w->dvars, &w->capdv, w->ndv + 1)) return -1;
        w->dvars[w->ndv++] = v;
    }
    w->ar_cl[w->nar] = c; w->ar_next[w->nar] = w->dhead[v];
    w->dhead[v] = (int32_t)w->nar++;
    return 0;
}

typedef struct {
    int64_t n_impl, cap;
    int32_t *ilit, *ireason;
    int64_t props, W, L, A, I;
} orc_out;

/* process the snapshot of var v's list. returns 1 on conflict, 0 otherwise, -1 on overflow */
static int scan_var(const orc_bcp *f, orc_ws *w, int32_t v, orc_out *o, int32_t *conflict_clause)
{
    const int32_t *lits = f->lits;
    int64_t n = 0;
    o->props++;
    /* snapshot: dynamic part newest first, then the initial list */
    for (int32_t e = w->dhead[v]; e != -1; e = w->ar_next[e]) {
        int32_t c = w->ar_cl[e];
        if (w->blk[c]) continue;
        int64_t b = f->coff[c];
        if ((lits[b + w->cw1[c]] >> 1) != v && (lits[b + w->cw2[c]] >> 1) != v) continue;
        if (grow32(&w->snap, &w->capsnap, n + 1)) return -1;
        w->snap[n++] = c;
    }
    for (int64_t k = f->w0off[v]; k < f->w0off[v + 1]; k++) {
        int32_t c = f->w0cl[k];
        if (w->blk[c]) continue;
        int64_t b = f->coff[c];
        if ((lits[b + w->cw1[c]] >> 1) != v && (lits[b + w->cw2[c]] >> 1) != v) continue;
        if (grow32(&w->snap, &w->capsnap, n + 1)) return -1;
        w->snap[n++] = c;
    }
    for (int64_t s = 0; s < n; s++) {
        int32_t c = w->snap[s];
        int64_t b = f->coff[c];
        int32_t k = (int32_t)(f->coff[c + 1] - b);
        int32_t i1 = w->cw1[c], i2 = w->cw2[c];
        int32_t l1 = lits[b + i1], l2 = lits[b + i2];
        int c1 = cons(w, l1), c2 = cons(w, l2);
        o->W++; o->L += k; o->A += 2;
        if (c1 && c2) continue;
        int pend = (!c1 && !c2) ? 2 : 1;
        int32_t f1 = -1, f2 = -1;
        for (int32_t idx = 0; pend > 0 && idx < k; idx++) {
            int32_t l = lits[b + idx];
            if (l != l1 && l != l2) {
                o->A++;
                if (cons(w, l)) {
                    if (f1 == -1) f1 = idx; else f2 = idx;
                    pend--;
                }
            }
        }
        int32_t unit = -1;
        if (c1 || c2) {
            if (f1 == -1) unit = lits[b + (c1 ? i1 : i2)];
            else {
                /* switch the inconsistent watch to f1 */
                if (touch(w, c)) return -1;
                if (!c1) w->cw1[c] = f1; else w->cw2[c] = f1;
                if (add_first(w, lits[b + f1] >> 1, c)) return -1;
                continue;
            }
        } else if (f1 != -1 && f2 != -1) {
            if (touch(w, c)) return -1;
            w->cw1[c] = f1;
            if (add_first(w, lits[b + f1] >> 1, c)) return -1;
            w->cw2[c] = f2;
            if (add_first(w, lits[b + f2] >> 1, c)) return -1;
            continue;
        } else if (f1 != -1) {
            unit = lits[b + f1];
        } else {
            if (touch(w, c)) return -1;
            w->blk[c] = 1;              /* handle_conflict blocks the clause */
            *conflict_clause = c;
            return 1;
        }
        /* handle_implication */
        if (w->val[unit >> 1] == 0) {
            if (o->n_impl >= o->cap) return -1;
            o->ilit[o->n_impl] = unit; o->ireason[o->n_impl] = c; o->n_impl++;
            w->val[unit >> 1] = (unit & 1) ? 1 : 2;
            o->I++;
        }
        if (touch(w, c)) return -1;
        w->blk[c] = 1;
    }
    return 0;
}

static void ws_reset(const orc_bcp *f, orc_ws *w, const int32_t *tl, int64_t tn, const orc_out *o)
{
    for (int64_t i = 0; i < tn; i++) w->val[tl[i] >> 1] = 0;
    for (int64_t i = 0; i < o->n_impl; i++) w->val[o->ilit[i] >> 1] = 0;
    for (int64_t i = 0; i < w->ntc; i++) {
        int32_t c = w->tclauses[i];
        w->touched[c] = 0; w->blk[c] = 0; w->cw1[c] = f->iw1[c]; w->cw2[c] = f->iw2[c];
    }
    w->ntc = 0;
    for (int64_t i = 0; i < w->ndv; i++) w->dhead[w->dvars[i]] = -1;
    w->ndv = 0; w->nar = 0;
}

/* One trail.  tl: internal literals.  Returns the status code. */
static int run_trail(const orc_bcp *f, orc_ws *w, const int32_t *tl, int64_t tn, orc_out *o,
                     int32_t *conflict_clause, int32_t *stop_index)
{
    int64_t assigned = 0;
    int status = ORC_BCP_NO_CONFLICT;
    *conflict_clause = -1; *stop_index = -1;
    /* a variable repeated with the same sign is simply propagated twice, as
     * the reference would; one given both signs is rejected */
    for (int64_t i = 0; i < tn; i++) {
        int32_t l = tl[i];
        int8_t want = (l & 1) ? 1 : 2;
        if (w->val[l >> 1] != 0 && w->val[l >> 1] != want) { status = ORC_BCP_BAD_TRAIL; break; }
        w->val[l >> 1] = want;
        assigned++;
    }
    if (status == ORC_BCP_NO_CONFLICT) {
        for (int64_t i = 0; i < tn && status == ORC_BCP_NO_CONFLICT; i++) {
            int64_t s = o->n_impl;
            int r = scan_var(f, w, tl[i] >> 1, o, conflict_clause);
            if (r != 0) { status = r > 0 ? ORC_BCP_CONFLICT : ORC_BCP_OVERFLOW; *stop_index = (int32_t)i; break; }
            /* depth-first over the implications of this call */
            int64_t depth = 0;
            if (o->n_impl > s) {
                if (w->capfr < 1) {
                    w->capfr = 1024;
                    w->fr_j = (int64_t *)malloc(sizeof(int64_t) * w->capfr);
                    w->fr_e = (int64_t *)malloc(sizeof(int64_t) * w->capfr);
                }
                w->fr_j[0] = s; w->fr_e[0] = o->n_impl; depth = 1;
            }
            while (depth > 0) {
                int64_t t = depth - 1;
                if (w->fr_j[t] < w->fr_e[t]) {
                    int32_t l = o->ilit[w->fr_j[t]++];
                    int64_t s2 = o->n_impl;
                    r = scan_var(f, w, l >> 1, o, conflict_clause);
                    if (r != 0) { status = r > 0 ? ORC_BCP_CONFLICT : ORC_BCP_OVERFLOW; *stop_index = (int32_t)i; break; }
                    if (o->n_impl > s2) {
                        if (depth == w->capfr) {
                            w->capfr *= 2;
                            w->fr_j = (int64_t *)realloc(w->fr_j, sizeof(int64_t) * w->capfr);
                            w->fr_e = (int64_t *)realloc(w->fr_e, sizeof(int64_t) * w->capfr);
                        }
                        w->fr_j[depth] = s2; w->fr_e[depth] = o->n_impl; depth++;
                    }
                } else {
                    depth--;
                }
            }
        }
    }
    /* undo the trail assignment: only the literals actually assigned */
    ws_reset(f, w, tl, assigned, o);
    return status;
}

/* ------------------------------------------------------------------ */
/* Full-scan clause evaluation (the reference's BASIC_SEARCH strategy):
 * every trail literal assigned, then sweeps over all clauses in index order,
 * each clause evaluated by clause_status -- true literal: satisfied; all
 * false: conflict, stop; exactly one unassigned (the last unassigned literal
 * it met) and the rest false: implied at once, visible to the clauses after
 * it -- repeated while a sweep adds implications.
 *     ConflictAnalysis/ConflictAnalyzer.cu:173-245 (propagate_all_clauses),
 *     :298-313 (clause_status), SATSolver/VariablesStateHandler.cu:180-206
 * Counters: [0] sweeps, [1] clause evaluations, [2] literals examined,
 * [3] assignment lookups (one per literal examined), [4] implications,
 * [5] trail literals.  stop_index = the sweep (0-based) that met the conflict. */
static int scan_trail(const orc_bcp *f, int8_t *val, const int32_t *tl, int64_t tn, orc_out *o,
                      int32_t *conflict_clause, int32_t *stop_index)
{
    int64_t assigned = 0;
    int status = ORC_BCP_NO_CONFLICT;
    *conflict_clause = -1; *stop_index = -1;
    for (int64_t i = 0; i < tn; i++) {
        int32_t l = tl[i];
        int8_t want = (l & 1) ? 1 : 2;
        if (val[l >> 1] != 0 && val[l >> 1] != want) { status = ORC_BCP_BAD_TRAIL; break; }
        val[l >> 1] = want;
        assigned++;
    }
    int64_t last = -1, sweep = 0;
    while (status == ORC_BCP_NO_CONFLICT && last != o->n_impl) {
        last = o->n_impl;
        o->props++;
        for (int64_t c = 0; c < f->n_clauses && status == ORC_BCP_NO_CONFLICT; c++) {
            int64_t b = f->coff[c], k = f->coff[c + 1] - b;
            int64_t unsat = 0;
            int32_t learnt = -1;
            int sat = 0;
            o->W++;
            for (int64_t i = 0; i < k; i++) {
                int32_t l = f->lits[b + i];
                int8_t a = val[l >> 1];
                o->L++; o->A++;
                if (a == 0) learnt = l;
                else if (a == ((l & 1) ? 1 : 2)) { sat = 1; break; }
                else unsat++;
            }
            if (sat) continue;
            if (unsat == k) {
                *conflict_clause = (int32_t)c;
                *stop_index = (int32_t)sweep;
                status = ORC_BCP_CONFLICT;
            } else if (unsat == k - 1) {
                if (o->n_impl >= o->cap) { status = ORC_BCP_OVERFLOW; *stop_index = (int32_t)sweep; break; }
                o->ilit[o->n_impl] = learnt; o->ireason[o->n_impl] = (int32_t)c; o->n_impl++;
                val[learnt >> 1] = (learnt & 1) ? 1 : 2;
                o->I++;
            }
        }
        sweep++;
    }
    for (int64_t i = 0; i < assigned; i++) val[tl[i] >> 1] = 0;
    for (int64_t i = 0; i < o->n_impl; i++) val[o->ilit[i] >> 1] = 0;
    return status;
}

typedef struct {
    const orc_bcp *f;
    const int32_t *trail; const int64_t *toff;
    int32_t n_trails, tid, nthreads;
    int64_t impl_cap;
    int32_t *status, *conflict_clause, *stop_index;
    int64_t *n_impl; int32_t *impl_lit, *impl_reason;
    int64_t *counters;
    int err;
    int scan;          /* 1: full-scan clause evaluation instead of BCP */
} orc_job;

static void *worker(void *arg)
{
    orc_job *j = (orc_job *)arg;
    const orc_bcp *f = j->f;
    orc_ws w;
    if (ws_init(&w, f)) { j->err = ORC_ERR_NOMEM; ws_free(&w); return NULL; }
    int32_t *tl = NULL; int64_t captl = 0;
    for (int32_t t = j->tid; t < j->n_trails; t += j->nthreads) {
        int64_t b = j->toff[t], tn = j->toff[t + 1] - b;
        if (grow32(&tl, &captl, tn + 1)) { j->err = ORC_ERR_NOMEM; break; }
        int bad = 0;
        for (int64_t i = 0; i < tn; i++) {
            int32_t d = j->trail[b + i];
            if (d == 0 || d > f->n_vars || d < -f->n_vars) { bad = 1; break; }
            tl[i] = lit_of_dimacs(d);
        }
        orc_out o;
        memset(&o, 0, sizeof(o));
        o.cap = j->impl_cap;
        o.ilit = j->impl_lit + (int64_t)t * j->impl_cap;
        o.ireason = j->impl_reason + (int64_t)t * j->impl_cap;
        int32_t cc = -1, si = -1;
        int st = bad ? ORC_BCP_BAD_TRAIL
                     : (j->scan ? scan_trail(f, w.val, tl, tn, &o, &cc, &si) : run_trail(f, &w, tl, tn, &o, &cc, &si));
        j->status[t] = st;
        j->conflict_clause[t] = cc;
        j->stop_index[t] = si;
        j->n_impl[t] = o.n_impl;
        for (int64_t i = 0; i < o.n_impl; i++) o.ilit[i] = dimacs_of_lit(o.ilit[i]);
        if (j->counters) {
            int64_t *cn = j->counters + (int64_t)t * 6;
            cn[0] = o.props; cn[1] = o.W; cn[2] = o.L; cn[3] = o.A; cn[4] = o.I;
            cn[5] = bad ? 0 : tn;
        }
    }
    free(tl);
    ws_free(&w);
    return NULL;
}

/* Runs every trail.  Outputs per trail t:
 *   status[t]          0 no conflict, 1 conflict, -1 capacity overflow, -2 bad trail
 *   conflict_clause[t] clause index or -1
 *   stop_index[t]      trail position whose propagation hit the conflict, or -1
 *   n_impl[t]          implied literals, written in order to
 *   impl_lit[t*cap ..] (DIMACS signed) and impl_reason[t*cap ..] (clause index)
 *   counters[t*6 ..]   props, watch entries, clause literals, assignment
 *                      lookups, implications, trail literals assigned   */
static int run_jobs(const orc_bcp *f, const int32_t *trail, const int64_t *toff, int32_t n_trails,
                    int32_t n_threads, int64_t impl_cap, int scan,
                    int32_t *status, int32_t *conflict_clause, int32_t *stop_index,
                    int64_t *n_impl, int32_t *impl_lit, int32_t *impl_reason, int64_t *counters);

int orc_bcp_run(const orc_bcp *f, const int32_t *trail, const int64_t *toff, int32_t n_trails,
                int32_t n_threads, int64_t impl_cap,
                int32_t *status, int32_t *conflict_clause, int32_t *stop_index,
                int64_t *n_impl, int32_t *impl_lit, int32_t *impl_reason, int64_t *counters)
{
    return run_jobs(f, trail, toff, n_trails, n_threads, impl_cap, 0, status, conflict_clause, stop_index,
                    n_impl, impl_lit, impl_reason, counters);
}

/* The same outputs for the full-scan strategy (scan_trail above). */
int orc_scan_run(const orc_bcp *f, const int32_t *trail, const int64_t *toff, int32_t n_trails,
                 int32_t n_threads, int64_t impl_cap,
                 int32_t *status, int32_t *conflict_clause, int32_t *stop_index,
                 int64_t *n_impl, int32_t *impl_lit, int32_t *impl_reason, int64_t *counters)
{
    return run_jobs(f, trail, toff, n_trails, n_threads, impl_cap, 1, status, conflict_clause, stop_index,
                    n_impl, impl_lit, impl_reason, counters);
}

static int run_jobs(const orc_bcp *f, const int32_t *trail, const int64_t *toff, int32_t n_trails,
                    int32_t n_threads, int64_t impl_cap, int scan,
                    int32_t *status, int32_t *conflict_clause, int32_t *stop_index,
                    int64_t *n_impl, int32_t *impl_lit, int32_t *impl_reason, int64_t *counters)
{
    if (!f || n_trails < 0 || impl_cap < 0) return ORC_ERR_ARG;
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_trails) n_threads = n_trails > 0 ? n_trails : 1;
    orc_job *jobs = (orc_job *)calloc(n_threads, sizeof(orc_job));
    pthread_t *th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
    int err = ORC_OK;
    for (int32_t i = 0; i < n_threads; i++) {
        orc_job *j = &jobs[i];
        j->f = f; j->trail = trail; j->toff = toff; j->n_trails = n_trails;
        j->tid = i; j->nthreads = n_threads; j->impl_cap = impl_cap;
        j->status = status; j->conflict_clause = conflict_clause; j->stop_index = stop_index;
        j->n_impl = n_impl; j->impl_lit = impl_lit; j->impl_reason = impl_reason;
        j->counters = counters;
        j->scan = scan;
    }
    if (n_threads == 1) {
        worker(&jobs[0]);
    } else {
        for (int32_t i = 0; i < n_threads; i++) pthread_create(&th[i], NULL, worker, &jobs[i]);
        for (int32_t i = 0; i < n_threads; i++) pthread_join(th[i], NULL);
    }
    for (int32_t i = 0; i < n_threads; i++) if (jobs[i].err) err = jobs[i].err;
    free(jobs); free(th);
    return err;
}
