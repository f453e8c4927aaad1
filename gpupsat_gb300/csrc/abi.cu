// C ABI: library info, error reporting, formula handles.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace gpsat {

namespace {
thread_local std::string g_last_error;
}

int set_error(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

int cuda_error(int cuda_code, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString((cudaError_t)cuda_code);
    cudaGetLastError();  // clear a sticky-free error so the next call starts clean
    return set_error(cuda_code == cudaErrorMemoryAllocation ? GPSAT_ERR_NOMEM : GPSAT_ERR_CUDA, m);
}

}  // namespace gpsat

using namespace gpsat;

extern "C" const char *gpsat_version(void) { return "gpsat 0.1.0 (sm_103a)"; }

extern "C" const char *gpsat_error_string(int code)
{
    switch (code) {
    case GPSAT_OK: return "ok";
    case GPSAT_ERR_ARG: return "bad argument";
    case GPSAT_ERR_CUDA: return "CUDA error";
    case GPSAT_ERR_NOMEM: return "out of memory";
    case GPSAT_ERR_FORMULA: return "invalid formula";
    case GPSAT_ERR_PARSE: return "DIMACS parse error";
    case GPSAT_ERR_CAPACITY: return "size exceeds a limit";
    case GPSAT_ERR_NODEVICE: return "no CUDA device";
    case GPSAT_ERR_TIMEOUT: return "device wait budget exhausted";
    case GPSAT_ERR_STATE: return "handle in the wrong state";
    default: return "unknown status code";
    }
}

extern "C" const char *gpsat_last_error(void) { return g_last_error.c_str(); }

extern "C" int gpsat_device_count(int32_t *count)
{
    if (!count) return set_error(GPSAT_ERR_ARG, "null count");
    int n = 0;
    cudaError_t err = cudaGetDeviceCount(&n);
    if (err != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return GPSAT_OK;
}

namespace gpsat {
namespace {

void formula_free_device(gpsat_formula *f)
{
    cudaFree(f->d_lits);
    cudaFree(f->d_coff);
    cudaFree(f->d_w0off);
    cudaFree(f->d_w0ent);
    f->d_lits = nullptr;
    f->d_coff = nullptr;
    f->d_w0off = nullptr;
    f->d_w0ent = nullptr;
}

template <class T>
bool upload(T **dst, const T *src, size_t n)
{
    if (cudaMalloc(dst, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return false;
    if (n && cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    return true;
}

}  // namespace
}  // namespace gpsat

namespace gpsat {

// Uploads the clause arena and initial watch lists to the device that is
// current on first use.  Host-side preparation never needs a GPU.
int formula_upload(gpsat_formula *f)
{
    if (f->uploaded) {
        cudaError_t err = cudaSetDevice(f->device);
        return err == cudaSuccess ? GPSAT_OK : cuda_error(err, "cudaSetDevice");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(GPSAT_ERR_NODEVICE, "no CUDA device visible");
    }
    cudaGetDevice(&f->device);
    const HostFormula &h = f->h;
    const int64_t m = h.n_clauses();
    std::vector<uint32_t> coff(m + 1);
    for (int64_t c = 0; c <= m; c++) coff[c] = (uint32_t)h.off[c];
    // one 32-byte entry per initial watch: {clause, literal offset, length,
    // (w1 << 16) | w2} then the clause's first four literals (0-padded)
    std::vector<int32_t> ent((size_t)h.w0off[h.n_vars] * 8);
    for (int32_t v = 0; v < h.n_vars; v++) {
        for (uint32_t k = h.w0off[v]; k < h.w0off[v + 1]; k++) {
            int32_t c = h.w0cl[k];
            int32_t *e = &ent[8 * (size_t)k];
            const int64_t b = h.off[c], len = h.off[c + 1] - b;
            e[0] = c;
            e[1] = (int32_t)b;
            e[2] = (int32_t)len;
            e[3] = (int32_t)(((uint32_t)h.w1[c] << 16) | (uint32_t)h.w2[c]);
            for (int i = 0; i < 4; i++) e[4 + i] = i < len ? h.lits[b + i] : 0;
        }
    }
    bool ok = upload(&f->d_lits, h.lits.data(), h.lits.size()) && upload(&f->d_coff, coff.data(), coff.size()) &&
              upload(&f->d_w0off, h.w0off.data(), h.w0off.size()) && upload(&f->d_w0ent, ent.data(), ent.size());
    if (!ok) {
        cudaError_t err = cudaGetLastError();
        formula_free_device(f);
        return cuda_error(err, "formula upload");
    }
    f->device_bytes = (int64_t)(h.lits.size() * 4 + coff.size() * 4 + h.w0off.size() * 4 + ent.size() * 4);
    f->uploaded = true;
    return GPSAT_OK;
}

}  // namespace gpsat

extern "C" int gpsat_formula_create(const int32_t *lits, const int64_t *offsets, int32_t n_vars, int64_t n_clauses,
                                    gpsat_formula **out)
{
    if (!out) return set_error(GPSAT_ERR_ARG, "null output handle");
    *out = nullptr;
    gpsat_formula *f = new gpsat_formula();
    int rc = prepare_formula(lits, offsets, n_vars, n_clauses, f->h);
    if (rc != GPSAT_OK) {
        delete f;
        return rc;
    }
    build_initial_watches(f->h);
    *out = f;
    return GPSAT_OK;
}

extern "C" int gpsat_formula_destroy(gpsat_formula *f)
{
    if (!f) return GPSAT_OK;
    if (f->uploaded) {
        cudaSetDevice(f->device);
        formula_free_device(f);
    }
    delete f;
    return GPSAT_OK;
}

extern "C" int gpsat_formula_info(const gpsat_formula *f, int32_t *n_vars, int64_t *n_clauses, int64_t *n_lits,
                                  int32_t *preproc_verdict, int64_t *n_solved)
{
    if (!f) return set_error(GPSAT_ERR_ARG, "null formula");
    if (n_vars) *n_vars = f->h.n_vars;
    if (n_clauses) *n_clauses = f->h.n_clauses();
    if (n_lits) *n_lits = (int64_t)f->h.lits.size();
    if (preproc_verdict) *preproc_verdict = f->h.verdict;
    if (n_solved) *n_solved = (int64_t)f->h.solved.size();
    return GPSAT_OK;
}

extern "C" int gpsat_formula_export(const gpsat_formula *f, int32_t *lits, int64_t *offsets, int32_t *solved_lits,
                                    int32_t *watch1, int32_t *watch2)
{
    if (!f) return set_error(GPSAT_ERR_ARG, "null formula");
    const HostFormula &h = f->h;
    if (lits)
        for (size_t i = 0; i < h.lits.size(); i++) lits[i] = dimacs_of_lit(h.lits[i]);
    if (offsets) std::memcpy(offsets, h.off.data(), h.off.size() * sizeof(int64_t));
    if (solved_lits)
        for (size_t i = 0; i < h.solved.size(); i++) solved_lits[i] = dimacs_of_lit(h.solved[i]);
    if (watch1 && !h.w1.empty()) std::memcpy(watch1, h.w1.data(), h.w1.size() * sizeof(int32_t));
    if (watch2 && !h.w2.empty()) std::memcpy(watch2, h.w2.data(), h.w2.size() * sizeof(int32_t));
    return GPSAT_OK;
}
