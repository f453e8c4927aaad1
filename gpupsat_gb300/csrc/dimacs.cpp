// DIMACS CNF reader.
//
// Accepts everything the reference's Boost.Spirit grammar accepts
// (reference FileManager/CnfReader.cpp:30-50: comment lines before a
// "p cnf <vars> <clauses>" header, then clauses of integers closed by 0) and,
// beyond it, comments between clauses, clauses spanning lines and a '%' end
// marker.  As in CnfManager::read_cnf (CnfReader.cpp:86-135) the variable
// count is the highest variable that occurs; the header's counts are
// reported back for the caller to compare.
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <string>

#include "internal.h"

using namespace gpsat;

namespace {

struct Cursor {
    const char *p, *e;
    int64_t line = 1;
    bool eof() const { return p >= e; }
    void skip_line()
    {
        while (p < e && *p != '\n') p++;
        if (p < e) {
            p++;
            line++;
        }
    }
    void skip_space()
    {
        while (p < e && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) {
            if (*p == '\n') line++;
            p++;
        }
    }
};

bool read_int(Cursor &c, long long &out)
{
    const char *s = c.p;
    bool neg = false;
    if (s < c.e && (*s == '-' || *s == '+')) {
        neg = *s == '-';
        s++;
    }
    if (s >= c.e || !std::isdigit((unsigned char)*s)) return false;
    long long v = 0;
    while (s < c.e && std::isdigit((unsigned char)*s)) {
        v = v * 10 + (*s - '0');
        if (v > INT32_MAX) return false;
        s++;
    }
    if (s < c.e && !(*s == ' ' || *s == '\t' || *s == '\r' || *s == '\n')) return false;
    c.p = s;
    out = neg ? -v : v;
    return true;
}

}  // namespace

// Two calls: with lits/offsets NULL it reports sizes only; then it fills them.
extern "C" int gpsat_dimacs_parse(const char *text, int64_t len, int32_t *n_vars, int64_t *n_clauses, int64_t *n_lits,
                                  int32_t *header_vars, int64_t *header_clauses, int32_t *lits, int64_t *offsets)
{
    if (!text || len < 0 || !n_vars || !n_clauses || !n_lits)
        return set_error(GPSAT_ERR_ARG, "gpsat_dimacs_parse: bad argument");
    Cursor c{text, text + len};
    long long hv = -1, hc = -1;
    // comments and blank lines, then the header
    for (;;) {
        c.skip_space();
        if (c.eof()) return set_error(GPSAT_ERR_PARSE, "missing 'p cnf' header");
        if (*c.p == 'c') {
            c.skip_line();
            continue;
        }
        if (*c.p == 'p') {
            c.p++;
            c.skip_space();
            if (c.e - c.p < 3 || std::strncmp(c.p, "cnf", 3) != 0)
                return set_error(GPSAT_ERR_PARSE, "line " + std::to_string(c.line) + ": expected 'p cnf'");
            c.p += 3;
            c.skip_space();
            if (!read_int(c, hv) || hv < 0)
                return set_error(GPSAT_ERR_PARSE, "line " + std::to_string(c.line) + ": bad variable count");
            c.skip_space();
            if (!read_int(c, hc) || hc < 0)
                return set_error(GPSAT_ERR_PARSE, "line " + std::to_string(c.line) + ": bad clause count");
            break;
        }
        return set_error(GPSAT_ERR_PARSE, "line " + std::to_string(c.line) + ": expected a comment or the header");
    }
    int64_t nc = 0, nl = 0, cur = 0;
    int32_t maxv = 0;
    for (;;) {
        c.skip_space();
        if (c.eof() || *c.p == '%') break;
        if (*c.p == 'c') {
            c.skip_line();
            continue;
        }
        long long x;
        if (!read_int(c, x))
            return set_error(GPSAT_ERR_PARSE, "line " + std::to_string(c.line) + ": expected an integer literal");
        if (x == 0) {
            // "0" alone is an empty clause, as the reference's grammar reads it
            // (the formula is then unsatisfiable)
            if (offsets) offsets[nc + 1] = nl;
            nc++;
            cur = 0;
            continue;
        }
        const int32_t v = (int32_t)(x > 0 ? x : -x);
        if (v > maxv) maxv = v;
        if (lits) lits[nl] = (int32_t)x;
        nl++;
        cur++;
    }
    if (cur != 0) return set_error(GPSAT_ERR_PARSE, "last clause is not terminated by 0");
    if (offsets) offsets[0] = 0;
    *n_vars = maxv;
    *n_clauses = nc;
    *n_lits = nl;
    if (header_vars) *header_vars = (int32_t)hv;
    if (header_clauses) *header_clauses = hc;
    return GPSAT_OK;
}
