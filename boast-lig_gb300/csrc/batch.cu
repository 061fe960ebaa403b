// Batched 3D operators over many grids of different sizes (orbitals with
// uneven localisation regions): each sweep stage of an operator is one
// persistent launch over the sweeps of all grids, the stages of a run are
// captured once in a CUDA graph, and an autotuner picks the engine and the
// sweep order per operator, kept in a JSON cache file.
//
// The per-grid work is exactly the single-grid plan (plan_magicfilter /
// plan_kinetic): stage k of the batch is step k of every grid's plan, with
// the grid's buffers packed back to back (x, y_mf, y_kin, w1, w2).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/libconv_gb300.h"
#include "lcg_plan.cuh"
#include "lcg_sweep.cuh"
#include "lcg_tc.cuh"

using namespace lcg;

namespace {

constexpr int kOps = 2;   // LIBCONV_BATCH_OP_MF, LIBCONV_BATCH_OP_KIN

struct Stage {
    int kind = 0, ntaps = 0;
    int src = 0, dst = 0, src2 = -1;         // plan buffer ids
    std::vector<Sweep> sw;                   // per grid, pointers unset
    std::vector<long long> off_src, off_dst, off_src2;   // per grid element offsets
    std::vector<Sweep> bound;                // per grid, pointers bound
    Sweep *d_desc = nullptr;
    long long *d_prefix = nullptr;
    long long units = 0;                     // tiles / blocks of the stage
    int grid = 0;                            // FP64 persistent grid
    TcFilter F;
    int *d_lineE = nullptr;                  // exact tensor-core sweeps: line exponents of all grids
    int exp_blocks = 0;                      // blocks per grid of their pass
};

struct OpConfig {
    bool enabled = false;
    int engine = LIBCONV_ENGINE_FP64_Q64;
    int order[3] = {-1, 0, 0};               // MF: order[0] = -1 -> rotating sweeps
    std::vector<Stage> stages;
};

}  // namespace

struct libconv_batch {
    int ngrids = 0, mode = LIBCONV_MODE_FP64, device = 0;
    std::vector<int> dims;                   // 3 per grid
    int mf_bc[3] = {0, 0, 0}, kin_bc[3] = {0, 0, 0};
    double kin_a[3] = {1, 1, 1}, kin_ax = 0.0;
    std::vector<long long> in_off, mf_off, kin_off, w_off;   // ngrids + 1 each
    double *w1 = nullptr, *w2 = nullptr;
    OpConfig op[kOps];
    bool tuned = false;
    // graph of the last bound configuration
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t graph_stream = nullptr;
    const double *bx = nullptr;
    double *by_mf = nullptr, *by_kin = nullptr;
    bool bound = false;
};

namespace {

int fail_arg(const char *msg) { return report(LIBCONV_EARG, msg); }

void free_stage(Stage &s) {
    if (s.d_desc) cudaFree(s.d_desc);
    if (s.d_prefix) cudaFree(s.d_prefix);
    if (s.d_lineE) cudaFree(s.d_lineE);
    s.d_desc = nullptr;
    s.d_prefix = nullptr;
    s.d_lineE = nullptr;
}

void drop_graph(libconv_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->bound = false;
}

bool engine_allowed(int mode, int engine) {
    if (engine == LIBCONV_ENGINE_TC) return mode != LIBCONV_MODE_FP64;
    return engine == LIBCONV_ENGINE_FP64_Q64 || engine == LIBCONV_ENGINE_FP64_Q32;
}

int scheme_of(int mode) {
    return mode == LIBCONV_MODE_TC_BF16X3 ? SCH_BF16X3
           : mode == LIBCONV_MODE_TC_TF32X3 ? SCH_TF32X3 : SCH_EXACT;
}

// Plan of grid g for operator o with order ord.
int grid_plan(const libconv_batch *b, int o, int g, const int *ord, Plan &P) {
    const int *n = &b->dims[3 * g];
    if (o == LIBCONV_BATCH_OP_MF) return plan_magicfilter(3, n, b->mf_bc, ord[0] < 0 ? nullptr : ord, P);
    return plan_kinetic(3, n, b->kin_bc, b->kin_a, b->kin_ax, ord, P);
}

// Build the stages of operator o for (engine, order): descriptors, tile /
// block prefix sums (device), filter operands.
int configure(libconv_batch *b, int o, int engine, const int *ord) {
    OpConfig &C = b->op[o];
    if (!engine_allowed(b->mode, engine))
        return report(LIBCONV_EMODE, "engine not available in this batch's compute mode");
    if (o == LIBCONV_BATCH_OP_KIN && ord[0] < 0) return fail_arg("kinetic needs an explicit order");
    for (Stage &s : C.stages) free_stage(s);
    C.stages.clear();
    drop_graph(b);
    const int G = b->ngrids;
    for (int g = 0; g < G; ++g) {
        Plan P;
        int rc = grid_plan(b, o, g, ord, P);
        if (rc) return rc;
        if (g == 0) C.stages.resize(P.steps.size());
        if (P.steps.size() != C.stages.size()) return fail_arg("grids with different plan shapes");
        for (size_t k = 0; k < P.steps.size(); ++k) {
            Stage &st = C.stages[k];
            const PlanStep &ps = P.steps[k];
            st.kind = ps.S.kind;
            st.ntaps = ps.S.ntaps;
            st.src = ps.src;
            st.dst = ps.dst;
            st.src2 = ps.src2;
            st.sw.push_back(ps.S);
            auto off = [&](int buf) -> long long {
                if (buf == B_X) return b->in_off[g];
                if (buf == B_Y) return o == LIBCONV_BATCH_OP_MF ? b->mf_off[g] : b->kin_off[g];
                return b->w_off[g];
            };
            st.off_src.push_back(off(ps.src));
            st.off_dst.push_back(off(ps.dst));
            st.off_src2.push_back(ps.src2 >= 0 ? off(ps.src2) : 0);
        }
    }
    const bool tc = engine == LIBCONV_ENGINE_TC;
    const int qc = engine == LIBCONV_ENGINE_FP64_Q32 ? 32 : 64;
    const double *ftab = filter_table();
    for (Stage &st : C.stages) {
        if (tc && !sweep_tc_batch_supported(st.kind, st.ntaps))
            return report(LIBCONV_EMODE, "no batched tensor-core sweep for this filter");
        std::vector<long long> prefix(G + 1, 0);
        for (int g = 0; g < G; ++g)
            prefix[g + 1] = prefix[g] + (tc ? sweep_tc_tiles(st.sw[g]) : sweep_fp64_batch_blocks(st.sw[g], qc));
        st.units = prefix[G];
        if (tc) {
            const Sweep &S0 = st.sw[0];
            const int sch = scheme_of(b->mode);
            const double a = S0.has_a ? S0.a : 1.0;
            if (sch == SCH_EXACT) tc_filter_digits(ftab + S0.ftab, S0.ntaps, a, st.F);
            else tc_filter_split(ftab + S0.ftab, S0.ntaps, a, sch, st.F);
            for (Sweep &S : st.sw) {
                S.has_a = 0;   // folded into the filter operands
                if (!tc_prepare(S)) return report(LIBCONV_EARG, "batch grid too large for the tensor-core sweep");
            }
            if (sch == SCH_EXACT) {
                // one pre-pass per stage writes every line's largest exponent
                long long lines = 0, most = 0;
                bool contiguous = false;
                for (Sweep &S : st.sw) {
                    S.le_off = lines;
                    const long long l = sweep_tc_lines(S);
                    lines += l;
                    most = l > most ? l : most;
                    contiguous |= S.nL == 1;
                }
                st.exp_blocks = line_exp_batch_blocks(most, contiguous);
                if (cudaMalloc(&st.d_lineE, sizeof(int) * (size_t)(lines > 0 ? lines : 1)) != cudaSuccess) {
                    cudaGetLastError();
                    return report(LIBCONV_ENOMEM, "batch line-exponent allocation failed");
                }
            }
        } else {
            st.grid = sweep_fp64_batch_grid(st.kind, st.ntaps, qc);
            if (st.grid <= 0) return report(LIBCONV_ECUDA, "no persistent grid for the FP64 sweep");
        }
        cudaError_t e = cudaMalloc(&st.d_desc, sizeof(Sweep) * G);
        if (e == cudaSuccess) e = cudaMalloc(&st.d_prefix, sizeof(long long) * (G + 1));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return report(LIBCONV_ENOMEM, "batch descriptor allocation failed");
        }
        e = cudaMemcpy(st.d_prefix, prefix.data(), sizeof(long long) * (G + 1), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return report_cuda(e, "upload tile prefix");
    }
    C.engine = engine;
    for (int i = 0; i < 3; ++i) C.order[i] = ord[i];
    return LIBCONV_OK;
}

// Bind the caller's buffers into the stage descriptors and upload them on st.
int bind(libconv_batch *b, const double *x, double *y_mf, double *y_kin, cudaStream_t stream) {
    double *base[4] = {const_cast<double *>(x), nullptr, b->w1, b->w2};
    for (int o = 0; o < kOps; ++o) {
        OpConfig &C = b->op[o];
        if (!C.enabled) continue;
        base[B_Y] = o == LIBCONV_BATCH_OP_MF ? y_mf : y_kin;
        for (Stage &st : C.stages) {
            st.bound = st.sw;
            for (int g = 0; g < b->ngrids; ++g) {
                Sweep &S = st.bound[g];
                S.x = base[st.src] + st.off_src[g];
                S.y = base[st.dst] + st.off_dst[g];
                S.x2 = st.src2 >= 0 ? base[st.src2] + st.off_src2[g] : nullptr;
            }
            cudaError_t e = cudaMemcpyAsync(st.d_desc, st.bound.data(), sizeof(Sweep) * b->ngrids,
                                            cudaMemcpyHostToDevice, stream);
            if (e != cudaSuccess) return report_cuda(e, "upload batch descriptors");
        }
    }
    b->bx = x;
    b->by_mf = y_mf;
    b->by_kin = y_kin;
    b->bound = true;
    return LIBCONV_OK;
}

int launch_op(libconv_batch *b, int o, int *status, cudaStream_t stream) {
    OpConfig &C = b->op[o];
    for (Stage &st : C.stages) {
        cudaError_t e;
        if (C.engine == LIBCONV_ENGINE_TC)
            e = launch_sweep_tc_batch(st.kind, st.ntaps, st.d_desc, st.d_prefix, b->ngrids, st.F,
                                      scheme_of(b->mode), status, st.d_lineE, st.exp_blocks, stream);
        else
            e = launch_sweep_fp64_batch(st.kind, st.ntaps, C.engine == LIBCONV_ENGINE_FP64_Q32 ? 32 : 64,
                                        st.d_desc, st.d_prefix, b->ngrids, st.grid, stream);
        if (e != cudaSuccess) return report_cuda(e, "batched sweep launch");
    }
    return LIBCONV_OK;
}

int launch_all(libconv_batch *b, int *status, cudaStream_t stream) {
    for (int o = 0; o < kOps; ++o) {
        if (!b->op[o].enabled) continue;
        int rc = launch_op(b, o, status, stream);
        if (rc) return rc;
    }
    return LIBCONV_OK;
}

// ---- tuning cache: a flat JSON object {"key": "engine,o0,o1,o2", ...} ----------
std::string cache_path() {
    const char *p = getenv("LIBCONV_GB300_TUNE_CACHE");
    if (p && *p) return p;
    const char *h = getenv("HOME");
    if (!h || !*h) return "";
    return std::string(h) + "/.cache/libconv_gb300_tune.json";
}

std::map<std::string, std::string> cache_load() {
    std::map<std::string, std::string> m;
    const std::string path = cache_path();
    if (path.empty()) return m;
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return m;
    std::string s;
    char buf[4096];
    size_t r;
    while ((r = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, r);
    fclose(f);
    std::vector<std::string> toks;
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] != '"') continue;
        size_t j = s.find('"', i + 1);
        if (j == std::string::npos) break;
        toks.push_back(s.substr(i + 1, j - i - 1));
        i = j;
    }
    for (size_t i = 0; i + 1 < toks.size(); i += 2) m[toks[i]] = toks[i + 1];
    return m;
}

void cache_store(const std::string &key, const std::string &val) {
    const std::string path = cache_path();
    if (path.empty()) return;
    std::map<std::string, std::string> m = cache_load();
    m[key] = val;
    // create missing parent directories
    for (size_t i = 1; i < path.size(); ++i)
        if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return;
    fprintf(f, "{\n");
    size_t i = 0;
    for (auto &kv : m) fprintf(f, "  \"%s\": \"%s\"%s\n", kv.first.c_str(), kv.second.c_str(), ++i < m.size() ? "," : "");
    fprintf(f, "}\n");
    fclose(f);
}

std::string cache_key(const libconv_batch *b, int o) {
    cudaDeviceProp prop;
    memset(&prop, 0, sizeof prop);
    cudaGetDeviceProperties(&prop, b->device);
    unsigned long long h = 1469598103934665603ull;   // FNV-1a over the grid shapes
    for (int v : b->dims) {
        h ^= (unsigned long long)(unsigned)v;
        h *= 1099511628211ull;
    }
    const int *bc = o == LIBCONV_BATCH_OP_MF ? b->mf_bc : b->kin_bc;
    char buf[512];
    snprintf(buf, sizeof buf, "%s|sm%d|mode%d|%s|bc%d,%d,%d|grids%d|%016llx", prop.name,
             prop.multiProcessorCount, b->mode, o == LIBCONV_BATCH_OP_MF ? "mf" : "kin", bc[0], bc[1],
             bc[2], b->ngrids, h);
    for (char *c = buf; *c; ++c)
        if (*c == '"' || *c == '\\') *c = '_';
    return buf;
}

std::string config_string(const OpConfig &C) {
    char buf[64];
    snprintf(buf, sizeof buf, "%d,%d,%d,%d", C.engine, C.order[0], C.order[1], C.order[2]);
    return buf;
}

bool parse_config(const std::string &s, int &engine, int ord[3]) {
    return sscanf(s.c_str(), "%d,%d,%d,%d", &engine, &ord[0], &ord[1], &ord[2]) == 4;
}

}  // namespace

extern "C" {

int libconv_batch_create(libconv_batch **out, int ngrids, const int *dims, const int *mf_bc,
                         const int *kin_bc, const double *kin_a, double kin_ax) {
    if (!out) return fail_arg("out must not be null");
    *out = nullptr;
    if (ngrids < 1 || !dims) return fail_arg("ngrids must be >= 1 and dims non-null");
    if (!mf_bc && !kin_bc) return fail_arg("at least one of mf_bc / kin_bc must be given");
    if (kin_bc && !kin_a) return fail_arg("kin_a must not be null with kin_bc");
    libconv_batch *b = new libconv_batch();
    b->ngrids = ngrids;
    b->mode = current_mode();
    cudaGetDevice(&b->device);
    b->dims.assign(dims, dims + 3 * ngrids);
    if (mf_bc) for (int i = 0; i < 3; ++i) b->mf_bc[i] = mf_bc[i];
    if (kin_bc) for (int i = 0; i < 3; ++i) b->kin_bc[i] = kin_bc[i], b->kin_a[i] = kin_a[i];
    b->kin_ax = kin_ax;
    b->op[LIBCONV_BATCH_OP_MF].enabled = mf_bc != nullptr;
    b->op[LIBCONV_BATCH_OP_KIN].enabled = kin_bc != nullptr;
    b->in_off.assign(ngrids + 1, 0);
    b->mf_off.assign(ngrids + 1, 0);
    b->kin_off.assign(ngrids + 1, 0);
    b->w_off.assign(ngrids + 1, 0);
    const int ref_order[3] = {-1, 0, 0}, nat[3] = {0, 1, 2};
    for (int g = 0; g < ngrids; ++g) {
        long long nin = 1, nmf = 1, ws = 0;
        for (int i = 0; i < 3; ++i) {
            const int n = dims[3 * g + i];
            if (n < 1) { delete b; return fail_arg("grid dimensions must be >= 1"); }
            nin *= n;
        }
        for (int o = 0; o < kOps; ++o) {
            if (!b->op[o].enabled) continue;
            // workspace: the largest w1/w2 over every sweep order the tuner may pick
            for (int v = -1; v < 6; ++v) {
                static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
                if (v < 0 && o == LIBCONV_BATCH_OP_KIN) continue;
                Plan P;
                int rc = grid_plan(b, o, g, v < 0 ? ref_order : perms[v], P);
                if (rc) { delete b; return rc; }
                ws = std::max<long long>(ws, (long long)std::max(P.elems[B_W1], P.elems[B_W2]));
                if (o == LIBCONV_BATCH_OP_MF) nmf = (long long)P.elems[B_Y];
            }
        }
        b->in_off[g + 1] = b->in_off[g] + nin;
        b->mf_off[g + 1] = b->mf_off[g] + (b->op[LIBCONV_BATCH_OP_MF].enabled ? nmf : 0);
        b->kin_off[g + 1] = b->kin_off[g] + (b->op[LIBCONV_BATCH_OP_KIN].enabled ? nin : 0);
        b->w_off[g + 1] = b->w_off[g] + ws;
    }
    const size_t wbytes = sizeof(double) * (size_t)std::max<long long>(b->w_off[ngrids], 1);
    if (cudaMalloc(&b->w1, wbytes) != cudaSuccess || cudaMalloc(&b->w2, wbytes) != cudaSuccess) {
        cudaGetLastError();
        libconv_batch_destroy(b);
        return report(LIBCONV_ENOMEM, "batch workspace allocation failed");
    }
    // configuration: the tuning cache, else the default engine of the mode
    std::map<std::string, std::string> cache = cache_load();
    bool all_cached = true;
    for (int o = 0; o < kOps; ++o) {
        if (!b->op[o].enabled) continue;
        int engine = b->mode == LIBCONV_MODE_FP64 ? LIBCONV_ENGINE_FP64_Q64 : LIBCONV_ENGINE_TC;
        int ord[3];
        memcpy(ord, o == LIBCONV_BATCH_OP_MF ? ref_order : nat, sizeof ord);
        auto it = cache.find(cache_key(b, o));
        if (it == cache.end() || !parse_config(it->second, engine, ord) ||
            !engine_allowed(b->mode, engine)) {
            all_cached = false;
            engine = b->mode == LIBCONV_MODE_FP64 ? LIBCONV_ENGINE_FP64_Q64 : LIBCONV_ENGINE_TC;
            memcpy(ord, o == LIBCONV_BATCH_OP_MF ? ref_order : nat, sizeof ord);
        }
        int rc = configure(b, o, engine, ord);
        if (rc) { libconv_batch_destroy(b); return rc; }
    }
    b->tuned = all_cached;
    *out = b;
    return LIBCONV_OK;
}

int libconv_batch_sizes(const libconv_batch *b, long long *in_elems, long long *mf_elems,
                        long long *kin_elems) {
    if (!b) return fail_arg("null batch");
    if (in_elems) *in_elems = b->in_off[b->ngrids];
    if (mf_elems) *mf_elems = b->mf_off[b->ngrids];
    if (kin_elems) *kin_elems = b->kin_off[b->ngrids];
    return LIBCONV_OK;
}

int libconv_batch_offsets(const libconv_batch *b, long long *in_off, long long *mf_off,
                          long long *kin_off) {
    if (!b) return fail_arg("null batch");
    const size_t n = sizeof(long long) * (b->ngrids + 1);
    if (in_off) memcpy(in_off, b->in_off.data(), n);
    if (mf_off) memcpy(mf_off, b->mf_off.data(), n);
    if (kin_off) memcpy(kin_off, b->kin_off.data(), n);
    return LIBCONV_OK;
}

int libconv_batch_set_config(libconv_batch *b, int op, int engine, const int *order) {
    if (!b || op < 0 || op >= kOps || !order) return fail_arg("bad batch / op / order");
    if (!b->op[op].enabled) return fail_arg("operator not enabled in this batch");
    if (!engine_allowed(b->mode, engine)) return report(LIBCONV_EMODE, "engine not available in this mode");
    return configure(b, op, engine, order);
}

int libconv_batch_get_config(const libconv_batch *b, int op, int *engine, int *order, int *tuned) {
    if (!b || op < 0 || op >= kOps) return fail_arg("bad batch / op");
    if (engine) *engine = b->op[op].engine;
    if (order) memcpy(order, b->op[op].order, 3 * sizeof(int));
    if (tuned) *tuned = b->tuned ? 1 : 0;
    return LIBCONV_OK;
}

int libconv_batch_run(libconv_batch *b, const double *x, double *y_mf, double *y_kin, void *stream) {
    if (!b || !x) return fail_arg("null batch or x");
    if (b->op[LIBCONV_BATCH_OP_MF].enabled && !y_mf) return fail_arg("y_mf must not be null");
    if (b->op[LIBCONV_BATCH_OP_KIN].enabled && !y_kin) return fail_arg("y_kin must not be null");
    int rc;
    int *status = device_status(rc);
    if (!status) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const bool same = b->bound && b->bx == x && b->by_mf == y_mf && b->by_kin == y_kin;
    if (!same) {
        if ((rc = bind(b, x, y_mf, y_kin, st))) return rc;
    }
    if (!st) return launch_all(b, status, st);   // the legacy stream cannot be captured
    if (!b->exec || b->graph_stream != st) {
        if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
        if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
        // one plain run first: one-time kernel set-up (shared-memory limits)
        // happens outside the capture; the captured run repeats the same work
        if ((rc = launch_all(b, status, st))) return rc;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return report_cuda(e, "begin graph capture");
        rc = launch_all(b, status, st);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(st, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        if (e != cudaSuccess) return report_cuda(e, "end graph capture");
        b->graph = g;
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) { b->exec = nullptr; return report_cuda(e, "graph instantiate"); }
        b->graph_stream = st;
    }
    cudaError_t e = cudaGraphLaunch(b->exec, st);
    if (e != cudaSuccess) return report_cuda(e, "graph launch");
    return LIBCONV_OK;
}

int libconv_batch_tune(libconv_batch *b, const double *x, double *y_mf, double *y_kin, void *stream) {
    if (!b || !x) return fail_arg("null batch or x");
    int rc;
    int *status = device_status(rc);
    if (!status) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const int engines[3] = {LIBCONV_ENGINE_TC, LIBCONV_ENGINE_FP64_Q64, LIBCONV_ENGINE_FP64_Q32};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int o = 0; o < kOps; ++o) {
        OpConfig &C = b->op[o];
        if (!C.enabled) continue;
        float best = 1e30f;
        int best_engine = C.engine, best_ord[3] = {C.order[0], C.order[1], C.order[2]};
        for (int ei = 0; ei < 3; ++ei) {
            const int engine = engines[ei];
            // split modes tune among the split tensor-core sweeps only
            if (!engine_allowed(b->mode, engine)) continue;
            if (engine != LIBCONV_ENGINE_TC && b->mode != LIBCONV_MODE_FP64 &&
                b->mode != LIBCONV_MODE_TC_EXACT)
                continue;
            for (int v = (o == LIBCONV_BATCH_OP_MF ? -1 : 0); v < 6; ++v) {
                const int ref[3] = {-1, 0, 0};
                const int *ord = v < 0 ? ref : perms[v];
                if ((rc = configure(b, o, engine, ord))) {
                    if (rc == LIBCONV_EMODE) continue;
                    cudaEventDestroy(e0); cudaEventDestroy(e1);
                    return rc;
                }
                if ((rc = bind(b, x, y_mf, y_kin, st))) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
                float ms = 0.f;
                for (int rep = 0; rep < 2; ++rep) {   // first run warms up
                    cudaEventRecord(e0, st);
                    if ((rc = launch_op(b, o, status, st))) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
                    cudaEventRecord(e1, st);
                    cudaError_t e = cudaEventSynchronize(e1);
                    if (e != cudaSuccess) { cudaEventDestroy(e0); cudaEventDestroy(e1); return report_cuda(e, "tuning run"); }
                    cudaEventElapsedTime(&ms, e0, e1);
                }
                if (ms < best) {
                    best = ms;
                    best_engine = engine;
                    memcpy(best_ord, ord, sizeof best_ord);
                }
            }
        }
        if ((rc = configure(b, o, best_engine, best_ord))) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
        cache_store(cache_key(b, o), config_string(C));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->tuned = true;
    b->bound = false;
    return LIBCONV_OK;
}

int libconv_batch_destroy(libconv_batch *b) {
    if (!b) return LIBCONV_OK;
    drop_graph(b);
    for (int o = 0; o < kOps; ++o)
        for (Stage &s : b->op[o].stages) free_stage(s);
    if (b->w1) cudaFree(b->w1);
    if (b->w2) cudaFree(b->w2);
    delete b;
    return LIBCONV_OK;
}

}  // extern "C"
