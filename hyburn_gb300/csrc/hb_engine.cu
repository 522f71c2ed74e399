// hb_engine.cu — host engine behind the C ABI of include/hyburn_gb300.h.
//
// Replaces BatchHybridEngine::from_config / run_sweep* (src/engine/batch_engine/engine.rs) for
// `--backend cuda`. The host side validates the descriptor with the reference's rules, lowers
// every projection into one device form (mean-field, diagonal, or CSR rows with packed per-edge
// delays), builds per-run parameter tables for the sweep, the BOLD emission schedule and the
// noise upload, and launches the simulation kernels of hb_kernels.cu. There is no host
// computation of the simulation itself and no fallback path.
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "hb_device.h"
#include "hyburn_gb300.h"

cudaError_t hb_launch_resident(int model, int fast, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem,
                               cudaStream_t st);
cudaError_t hb_launch_bold_batch_mean(const DevBold& bold, int m, int n_windows, int B, float* means, cudaStream_t st);
int hb_resident_smem_budget(int model, int fast, int threads);
cudaError_t hb_launch_pipe_512(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_pipe_1024(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
int hb_pipe_budget_512(int model, int pre);
int hb_pipe_budget_1024(int model, int pre);
cudaError_t hb_launch_stream_1(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_stream_2(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
cudaError_t hb_launch_stream_4(int model, int pre, const DevNet* d_net, const RunArgs& a, int B, int threads, size_t smem, cudaStream_t st);
int hb_stream_budget_1(int model, int pre);
int hb_stream_budget_2(int model, int pre);
int hb_stream_budget_4(int model, int pre);
int hb_stream_clusters_1(int model, int pre, int C, int threads, size_t smem);
int hb_stream_clusters_2(int model, int pre, int C, int threads, size_t smem);
int hb_stream_clusters_4(int model, int pre, int C, int threads, size_t smem);
cudaError_t hb_launch_single(int model, int m, const DevNet* d_net, const RunArgs& a, int B, cudaStream_t st);
// hb_dense_tc.cu
int hb_dense_tc_tmem_columns(int model, int nm);
void hb_dense_tc_tiles(const float* w, int nm, int NP, int KP, float* out);
cudaError_t hb_launch_dense_tc(int model, const DevNet* d_net, const RunArgs& a, int B, const float* wtiles, int NP, int KP,
                               int NPN, cudaStream_t st);
cudaError_t hb_launch_stream_queue_1(const StreamJob* d_jobs, int n_jobs, int n_items, int* counter, int blocks, int threads, size_t smem, int C, cudaStream_t st);
int hb_stream_queue_grid_1(int threads, size_t smem, int C);
cudaError_t hb_launch_stream_queue_2(const StreamJob* d_jobs, int n_jobs, int n_items, int* counter, int blocks, int threads, size_t smem, int C, cudaStream_t st);
int hb_stream_queue_grid_2(int threads, size_t smem, int C);
cudaError_t hb_launch_stream_queue_4(const StreamJob* d_jobs, int n_jobs, int n_items, int* counter, int blocks, int threads, size_t smem, int C, cudaStream_t st);
int hb_stream_queue_grid_4(int threads, size_t smem, int C);
int hb_stream_queue_budget_1();
int hb_stream_queue_budget_2();
int hb_stream_queue_budget_4();
cudaError_t hb_launch_adjoint(const DevNet* d_net, const HbAdjointLaunch& L, int phase, cudaStream_t st);
// hb_io.cu
hb_status hb_io_make_dirs(const std::string& dir);
hb_status hb_io_write_npy(const std::string& path, const float* data, const std::vector<int64_t>& shape);

namespace {

thread_local std::string g_err;

hb_status fail(hb_status st, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

#define CUDA_TRY(x)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess) return fail(HB_ERR_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_)); \
    } while (0)

// ---- model registry (src/config.rs:43-72); the six batch-native models are supported ----
struct ModelInfo { const char* name; int nvar, ncvar, nparams, native_sweep, cvar0; };
const ModelInfo k_models[6] = {
    {"Generic2dOscillator", 2, 1, 12, 1, 0}, {"MontbrioPazoRoxin", 2, 2, 7, 4, 0}, {"ReducedWongWang", 1, 1, 8, 7, 0},
    {"Kuramoto", 1, 1, 1, 0, 0},             {"JansenRit", 6, 1, 13, 12, 1},     {"WilsonCowan", 2, 1, 22, 18, 0},
};
const char* k_other_models[] = {
    "Linear", "SupHopf", "Hopfield", "CoombesByrne2D", "CoombesByrne", "GastSchmidtKnoscheSD", "GastSchmidtKnoscheSF",
    "LarterBreakspear", "Epileptor2D", "Epileptor", "ReducedWongWangExcInh", "DecoBalancedExcInh", "EpileptorCodim3",
    "EpileptorCodim3SlowMod", "EpileptorRestingState", "ZetterbergJansen", "ReducedSetFitzHughNagumo",
    "ReducedSetHindmarshRose", "DumontGutkin", "ZerlautAdaptationFirstOrder", "ZerlautAdaptationSecondOrder", "KIonEx"};
const int k_other_nvar[] = {1, 2, 2, 2, 4, 4, 4, 3, 2, 6, 2, 2, 3, 5, 8, 12, 4, 6, 8, 5, 8, 5};
const int k_other_ncvar[] = {1, 2, 2, 2, 4, 4, 4, 1, 1, 2, 1, 1, 1, 1, 3, 1, 2, 2, 4, 1, 1, 1};
const int k_other_np[] = {1, 2, 3, 4, 5, 9, 9, 32, 12, 17, 19, 20, 13, 27, 28, 18, 8, 12, 14, 50, 50, 14};

// the registry's names in its order, comma-separated: the list SimConfig::validate prints for an
// unknown model (config.rs:297-303)
std::string known_models() {
    std::string out;
    for (const ModelInfo& mi : k_models) out += (out.empty() ? "" : ", ") + std::string(mi.name);
    for (const char* n : k_other_models) out += ", " + std::string(n);
    return out;
}

int model_id(const char* name) {
    if (!name) return -1;
    for (int i = 0; i < 6; i++)
        if (strcmp(name, k_models[i].name) == 0) return i;
    return -1;
}
bool is_other_model(const char* name) {
    if (!name) return false;
    for (const char* m : k_other_models)
        if (strcmp(name, m) == 0) return true;
    return false;
}

// ---- coupling functions: CouplingFnConfig::from_name_and_params (coupling.rs:114-202) ----
struct Cfn {
    int kind = HBC_LINEAR;
    float a = 1, b = 0, cmin = 0, cmax = 0, mid = 0, sigma = 1, r = 0, e0 = 0, v0 = 0;
    int classic = 0;
    float h = 1, q = 1, g = 1, p = 1, theta = 0.5f;
    int dynamic = 0, global_t = 0;
};

bool cfn_parse(const char* name, const float* cp, int n, Cfn& f) {
    f = Cfn();
    auto P = [&](int i, float d) { return n > i ? cp[i] : d; };
    if (!name) return false;
    if (!strcmp(name, "Linear")) { f.kind = HBC_LINEAR; f.a = P(0, 1.0f); f.b = P(1, 0.0f); }
    else if (!strcmp(name, "Sigmoidal")) {
        f.kind = HBC_SIGMOIDAL;
        if (n >= 5) { f.cmin = cp[0]; f.cmax = cp[1]; f.mid = cp[2]; f.a = cp[3]; f.sigma = cp[4]; }
        else { f.cmin = -1.0f; f.cmax = P(0, 1.0f); f.mid = P(1, 0.0f); f.a = 1.0f; f.sigma = P(2, 1.0f); }
    } else if (!strcmp(name, "Difference")) { f.kind = HBC_DIFFERENCE; f.a = P(0, 1.0f); }
    else if (!strcmp(name, "Kuramoto")) { f.kind = HBC_KURAMOTO; f.a = P(0, 1.0f); }
    else if (!strcmp(name, "ScaledLinear")) { f.kind = HBC_SCALED_LINEAR; f.a = P(0, 1.0f); f.b = P(1, 0.0f); }
    else if (!strcmp(name, "HyperbolicTangent")) { f.kind = HBC_TANH; f.a = P(0, 1.0f); f.b = P(1, 1.0f); f.mid = P(2, 0.0f); f.sigma = P(3, 1.0f); }
    else if (!strcmp(name, "SigmoidalJansenRit")) {
        f.kind = HBC_SJR;
        if (n >= 5) { f.a = cp[0]; f.classic = 1; f.cmin = cp[1]; f.cmax = cp[2]; f.r = cp[3]; f.mid = cp[4]; f.e0 = 0.005f; f.v0 = 6.0f; }
        else { f.a = P(0, 1.0f); f.classic = 0; f.cmin = 0.0f; f.cmax = 0.005f; f.r = P(2, 0.56f); f.mid = 6.0f; f.e0 = P(1, 0.005f); f.v0 = P(3, 6.0f); }
    } else if (!strcmp(name, "PreSigmoidal")) {
        f.kind = HBC_PRESIG; f.h = P(0, 1.0f); f.q = P(1, 1.0f); f.g = P(2, 1.0f); f.p = P(3, 1.0f); f.theta = P(4, 0.5f);
        f.dynamic = (n > 5 && cp[5] != 0.0f); f.global_t = (n > 6 && cp[6] != 0.0f);
    } else return false;
    return true;
}

struct HostSub {
    int model, nnodes, nmodes, nm, nvar, ncvar, nparams;
    std::vector<float> params, x0;
    std::vector<float> node_params;  // [nm][nparams] or [B][nm][nparams] (extension), empty for none
    bool node_pp = false;            // node_params holds one table per sweep point
};

enum { W_MEAN = 0, W_DIAG = 1, W_SPARSE = 2 };

struct HostProj {
    int src, tgt, kind, dmode, delay, nsrc, ntgt;
    std::string cf_name;
    std::vector<float> cf_params;
    int diff_mode = 0;   // 1: Difference became Linear{a,0}; 2: Difference with rowsums
    Cfn cf;              // resolved with the configured parameters
    float w = 0;
    std::vector<int> rowptr;
    std::vector<uint32_t> edges;
    std::vector<int> eoff;
    std::vector<float> ew, rowsums;
    int maxd = 0;
    int direct = 0, ncm = 0, cm_s[4] = {0, 0, 0, 0}, cm_cpl[4] = {0, 0, 0, 0};
    int ncv = 1, pc = 1, oc = 1, pre_cpu = 0;
    // device copies
    int* d_rowptr = nullptr;
    uint32_t* d_edges = nullptr;
    int* d_eoff = nullptr;
    float* d_ew = nullptr;
    float* d_rowsums = nullptr;
    float* d_cp_pp = nullptr;
    size_t cp_pp_cap = 0;
};

Cfn resolve_cfn(const HostProj& hp, const float* params, int n) {
    Cfn f;
    if (!cfn_parse(hp.cf_name.c_str(), params, n, f)) {
        f = Cfn();  // engine.rs:277-279: unknown names fall back to Linear{a:1,b:0}
        f.kind = HBC_LINEAR; f.a = 1.0f; f.b = 0.0f;
    }
    if (f.kind == HBC_DIFFERENCE && hp.diff_mode == 1) {
        float a = f.a;
        f = Cfn();
        f.kind = HBC_LINEAR; f.a = a; f.b = 0.0f;
    }
    return f;
}

void cfn_to_cp(const Cfn& f, int n_src, float* cp) {
    for (int i = 0; i < HB_NCP; i++) cp[i] = 0.0f;
    switch (f.kind) {
    case HBC_LINEAR: case HBC_SCALED_LINEAR: cp[0] = f.a; cp[1] = f.b; break;
    case HBC_SIGMOIDAL: cp[0] = f.cmin; cp[1] = f.cmax; cp[2] = f.mid; cp[3] = f.a; cp[4] = f.sigma; break;
    case HBC_DIFFERENCE: cp[0] = f.a; break;
    case HBC_KURAMOTO: cp[0] = f.a; cp[1] = f.a / (float)n_src; break;
    case HBC_TANH: cp[0] = f.a; cp[1] = f.b; cp[2] = f.mid; cp[3] = f.sigma; break;
    case HBC_SJR: cp[0] = f.a; cp[1] = (float)f.classic; cp[2] = f.cmin; cp[3] = f.cmax; cp[4] = f.r; cp[5] = f.mid; cp[6] = f.e0; cp[7] = f.v0; break;
    case HBC_PRESIG: cp[0] = f.h; cp[1] = f.q; cp[2] = f.g; cp[3] = f.p; cp[4] = f.theta; cp[5] = (float)f.dynamic; break;
    }
}

int parse_cvar_map(const char* s, int* ps, int* pt, int maxn) {
    int n = 0;
    std::string str = s ? s : "0:0";
    size_t pos = 0;
    while (pos <= str.size() && n < maxn) {
        size_t e = str.find(',', pos);
        std::string part = str.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
        size_t a = part.find_first_not_of(" \t"), z = part.find_last_not_of(" \t");
        if (a != std::string::npos) {
            part = part.substr(a, z - a + 1);
            int v1 = 0, v2 = 0;
            size_t c = part.find(':');
            if (c != std::string::npos && part.find(':', c + 1) == std::string::npos) {
                char* endp;
                std::string l = part.substr(0, c), r = part.substr(c + 1);
                long x1 = strtol(l.c_str(), &endp, 10);
                if (*endp || l.empty() || x1 < 0) x1 = 0;
                long x2 = strtol(r.c_str(), &endp, 10);
                if (*endp || r.empty() || x2 < 0) x2 = 0;
                v1 = (int)x1; v2 = (int)x2;
            }
            ps[n] = v1; pt[n] = v2; n++;
        }
        if (e == std::string::npos) break;
        pos = e + 1;
    }
    return n;
}

// a device allocation owned by its holder (freed on destruction; move-only)
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DBuf() { release(); }
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr; n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = std::max<size_t>(count, 1);
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

struct BoldHost {
    int period;
    double tr;
    std::vector<double> times;   // all BOLD sample times so far (ms)
    int64_t n_out = 0;           // TR outputs produced so far
    std::vector<float> out;      // batch mean: [n_out][N0]; per point: [B][n_out][N0]
    DBuf<float> bw, acc, win, out_run;
    DBuf<BoldEmit> emit;
};

struct RunTables {
    std::vector<std::vector<float>> params;  // per sub [B][PSTRIDE]
    std::vector<std::vector<float>> node_params;  // per sub [Bn][nm][PSTRIDE] (Bn = 1 or B), empty without node rows
    std::vector<int> node_pp;                // per sub: node table per point (Bn = B)
    std::vector<int> sweep_form;
    std::vector<std::vector<float>> cp_pp;   // per proj [B][NCP] or empty
    std::vector<float> param_values;
};

}  // namespace

struct hb_engine {
    int B = 0;
    double dt_ms = 0;
    int integrator = 0;
    uint32_t flags = 0;
    std::vector<float> nsig;
    std::vector<HostSub> subs;
    std::vector<HostProj> projs;
    std::vector<hb_bold_desc> bold_cfg;
    bool bold_removed = false;   // run_sweep_multi drops the monitors (engine.rs:1330-1333)
    int H = 0, R = 0, cols = 0, state_len = 0, noise_row = 0, threads = 0, n_mean = 0;
    int kernel_model = -1;   // the model all subnetworks share, or -1
    int sync_every = 1;      // barrier interval of the specialised kernel (<= smallest delay)
    int dmin = 0;            // smallest edge delay of a one-projection network (0: not applicable)
    DevNet net;
    DevNet* d_net = nullptr;
    DBuf<float> state, x0, tavg, ring, noise, prep_noise, traj, means;
    DBuf<float> dtraj;          // HB_RUN_DEVICE_TRAJECTORY: [dtraj_steps][B][state_len] of the last run
    int64_t dtraj_steps = 0;    // 0: the last run kept no device trajectory
    float* cs_out = nullptr;    // the order-parameter adjoint's request for the coupling sums of every step
    DBuf<float> fe_fc, fe_feat, fe_fcd, fe_fcds, fe_ut;  // hb_engine_fc_features outputs and workspace
    DBuf<double> fe_part, fe_mv;
    // streamed-history kernel: its own ring [B][nm][rp + K][channels]; the layout of the history
    // a run leaves behind (0: time-major ring, 1: streamed) must match the next run's kernel
    DBuf<float> sring;
    int hist_layout = 0, hist_rp = 0;
    int hist_R = 0;           // ring length (slots) of the time-major history the last run left
    std::vector<DBuf<float>> d_params;
    std::vector<DBuf<float>> d_node_params;
    DBuf<float> dtc;            // the tensor-core path's W in its shared-memory layout (hi and lo TF32 parts)
    DBuf<int> porder;           // producer node order of the last run's pipeline / streamed-history kernel
    DBuf<int> flags_buf;
    std::vector<BoldHost> bold;
    cudaStream_t own_stream = nullptr, user_stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int64_t step = 0;
    double last_ms = 0;
    int64_t last_launches = 0;
    int last_kind = 0;
    // prepared run
    bool prepared = false;
    RunTables prep_tables;
    int64_t prep_steps = 0;
    uint32_t prep_flags = 0;
    int64_t prep_noise_len = 0;

    cudaStream_t stream() const { return user_stream ? user_stream : own_stream; }
};

struct hb_result {
    int n_sweep = 0;
    double elapsed_ms = 0;
    std::vector<float> params;
    std::vector<std::vector<float>> tavg, fin, traj;
    bool has_traj = false;
    std::vector<std::vector<float>> bold;
    int n_bold = 0;
};

namespace {

int eff_integrator(const hb_engine* e, int model) {
    bool use_heun = (e->flags & HB_SEM_HYBRID_INTEGRATOR) ? (model == HBM_G2DO) : (e->integrator == HB_INT_HEUN);
    if (use_heun) return HBI_HEUN_DET;
    switch (e->integrator) {
    case HB_INT_EULER: return HBI_EULER;
    case HB_INT_EULER_STOCHASTIC: return HBI_EULER_STOCH;
    case HB_INT_HEUN_STOCHASTIC: return HBI_HEUN_STOCH;
    case HB_INT_RK4: return HBI_RK4;
    case HB_INT_RK4_STOCHASTIC: return HBI_RK4_STOCH;
    default: return HBI_EULER;  // `_ =>` arm: Heun under hybrid integration for non-oscillators
    }
}

// shared memory of the streamed-history kernel's parameter rows [nm][params used] (several nodes per
// consumer thread only), with the alignment padding before them
size_t stream_prm_bytes(int model, int nm, int npt) {
    static const int used[6] = {12, 7, 8, 1, 13, 26};  // c_nparams_used of hb_models.cuh, by model id
    if (npt <= 1 || model < 0 || model > 5) return 0;
    return (size_t)nm * used[model] * 4 + 16;
}

bool is_stochastic(int integ) { return integ == HBI_EULER_STOCH || integ == HBI_HEUN_STOCH || integ == HBI_RK4_STOCH; }

void fill_derived(int model, float* row) {
    if (model == HBM_WC) {
        row[HB_D_WC_SIG_E_OFF] = 1.0f / (1.0f + expf(row[6] * row[7]));
        row[HB_D_WC_SIG_I_OFF] = 1.0f / (1.0f + expf(row[10] * row[11]));
    }
}

// per-run tables for a sweep (engine.rs:477-535 single, 862-940 multi)
hb_status build_tables(hb_engine* e, const hb_sweep_point* dims, int n_dims, bool multi, RunTables& T) {
    const int B = e->B;
    const int ns = (int)e->subs.size(), np = (int)e->projs.size();
    T.params.assign(ns, std::vector<float>((size_t)B * HB_PSTRIDE, 0.0f));
    T.sweep_form.assign(ns, 0);
    T.cp_pp.assign(np, std::vector<float>());
    for (int i = 0; i < ns; i++)
        for (int b = 0; b < B; b++) {
            float* row = &T.params[i][(size_t)b * HB_PSTRIDE];
            for (int k = 0; k < e->subs[i].nparams; k++) row[k] = e->subs[i].params[k];
        }
    std::vector<int> cnt(ns, 0);
    std::vector<char> proj_swept(np, 0);
    for (int d = 0; d < n_dims; d++) {
        int si = dims[d].sub_idx;
        if (si >= ns || si < -np) return fail(HB_ERR_INVALID_CONFIG, "subnetwork index %d out of range", si);
        if (si >= 0) cnt[si]++;
        else {
            int p = -1 - si;
            if (dims[d].param_idx < 0 || dims[d].param_idx >= (int)e->projs[p].cf_params.size())
                return fail(HB_ERR_INVALID_CONFIG, "projection %d has %d coupling params, cannot sweep index %d", p,
                            (int)e->projs[p].cf_params.size(), dims[d].param_idx);
            proj_swept[p] = 1;
        }
    }
    // mode per subnetwork: 0 none, 1 native sweep form, 2 per-point parameters (dfun.rs:39-45, 99-133)
    std::vector<int> mode(ns, 0);
    for (int i = 0; i < ns; i++) {
        if (!cnt[i]) continue;
        if (cnt[i] == 1) {
            int d0 = 0;
            while (dims[d0].sub_idx != i) d0++;
            mode[i] = (dims[d0].param_idx == k_models[e->subs[i].model].native_sweep) ? 1 : 0;
        } else mode[i] = 2;
        T.sweep_form[i] = (mode[i] == 1);
    }
    for (int p = 0; p < np; p++)
        if (proj_swept[p]) T.cp_pp[p].assign((size_t)B * HB_NCP, 0.0f);
    T.param_values.clear();
    std::vector<float> vals(n_dims);
    for (int b = 0; b < B; b++) {
        int64_t rem = b;
        for (int d = n_dims - 1; d >= 0; d--) {
            int nv = multi ? dims[d].n_values : B;
            int64_t idx = multi ? rem % nv : b;
            if (multi) rem /= nv;
            vals[d] = dims[d].values[idx];
        }
        for (int d = 0; d < n_dims; d++) T.param_values.push_back(vals[d]);
        for (int d = 0; d < n_dims; d++) {
            int si = dims[d].sub_idx;
            if (si < 0 || mode[si] == 0) continue;
            if (dims[d].param_idx >= 0 && dims[d].param_idx < e->subs[si].nparams)
                T.params[si][(size_t)b * HB_PSTRIDE + dims[d].param_idx] = vals[d];
        }
        for (int p = 0; p < np; p++) {
            if (!proj_swept[p]) continue;
            HostProj& hp = e->projs[p];
            std::vector<float> prm = hp.cf_params;
            for (int d = 0; d < n_dims; d++)
                if (dims[d].sub_idx == -1 - p) prm[dims[d].param_idx] = vals[d];
            Cfn f = resolve_cfn(hp, prm.data(), (int)prm.size());
            cfn_to_cp(f, hp.nsrc, &T.cp_pp[p][(size_t)b * HB_NCP]);
        }
    }
    for (int i = 0; i < ns; i++)
        for (int b = 0; b < B; b++) fill_derived(e->subs[i].model, &T.params[i][(size_t)b * HB_PSTRIDE]);
    // node rows (extension): the node's row, then the swept values of point b as above
    T.node_params.assign(ns, std::vector<float>());
    T.node_pp.assign(ns, 0);
    for (int i = 0; i < ns; i++) {
        const HostSub& S = e->subs[i];
        if (S.node_params.empty()) continue;
        const int Bn = (S.node_pp || mode[i] != 0) ? B : 1;
        T.node_pp[i] = Bn == B ? 1 : 0;
        T.node_params[i].assign((size_t)Bn * S.nm * HB_PSTRIDE, 0.0f);
        for (int b = 0; b < Bn; b++) {
            const float* src_tab = S.node_params.data() + (S.node_pp ? (size_t)b * S.nm * S.nparams : 0);
            for (int n = 0; n < S.nm; n++) {
                float* row = &T.node_params[i][((size_t)b * S.nm + n) * HB_PSTRIDE];
                for (int k = 0; k < S.nparams; k++) row[k] = src_tab[(size_t)n * S.nparams + k];
                if (mode[i] != 0) {
                    const float* pr = &T.params[i][(size_t)b * HB_PSTRIDE];
                    for (int d = 0; d < n_dims; d++)
                        if (dims[d].sub_idx == i && dims[d].param_idx >= 0 && dims[d].param_idx < S.nparams)
                            row[dims[d].param_idx] = pr[dims[d].param_idx];
                }
                fill_derived(S.model, row);
            }
        }
    }
    return HB_OK;
}

// BOLD sample times and TR outputs of a run of n_steps (bold_monitor.rs:72-227); fills the emit
// schedule and returns the number of new outputs
int64_t bold_schedule(const hb_engine* e, BoldHost& bh, int64_t n_steps, std::vector<BoldEmit>& emit,
                      int& n_full, int& partial, std::vector<double>& new_times) {
    const double dt_bold = e->dt_ms * (double)bh.period;
    const double tr_ms = bh.tr * 1000.0;
    n_full = (int)(n_steps / bh.period);
    partial = (int)(n_steps % bh.period);
    int64_t n_prev = (int64_t)bh.times.size();
    new_times.clear();
    for (int k = 0; k < n_full; k++) new_times.push_back((double)(n_prev + k) * dt_bold + dt_bold);
    if (partial > 0) new_times.push_back((double)(n_prev + n_full) * dt_bold + e->dt_ms * (double)partial);
    std::vector<double> times = bh.times;
    times.insert(times.end(), new_times.begin(), new_times.end());
    emit.clear();
    const int64_t ns = (int64_t)times.size();
    if (ns == 0) return 0;
    if (tr_ms <= 0.0 || std::fabs(tr_ms - dt_bold) < 1e-6) {
        // native sampling: every sample is an output
        for (int64_t k = n_prev; k < ns; k++) emit.push_back({(int)(k - n_prev), (int)(k - n_prev), 0, 0.0f});
        return ns - n_prev;
    }
    double max_t = times.back();
    int64_t n_out = max_t >= tr_ms ? (int64_t)std::floor(max_t / tr_ms) : 0;
    int64_t j0 = bh.n_out;
    for (int64_t j = j0; j < n_out; j++) {
        double tt = (double)(j + 1) * tr_ms;
        BoldEmit em;
        em.out = (int)(j - j0);
        if (tt <= times[0]) { em.k = 0; em.interp = 0; em.w = 0; }
        else {
            int64_t idx = 0;
            for (int64_t k = 1; k < ns; k++) {
                if (times[k] > tt) { idx = k - 1; break; }
                idx = k;
            }
            if (idx + 1 >= ns) { em.k = (int)idx; em.interp = 0; em.w = 0; }
            else {
                double t0 = times[idx], t1 = times[idx + 1];
                double w = std::fabs(t1 - t0) < 1e-12 ? 0.0 : (tt - t0) / (t1 - t0);
                w = std::min(1.0, std::max(0.0, w));
                em.k = (int)(idx + 1); em.interp = 1; em.w = (float)w;
            }
        }
        em.k -= (int)n_prev;  // run-local sample index
        emit.push_back(em);
    }
    std::stable_sort(emit.begin(), emit.end(), [](const BoldEmit& a, const BoldEmit& b) { return a.k < b.k; });
    return n_out - j0;
}

hb_status upload_net(hb_engine* e, const RunTables& T) {
    cudaStream_t st = e->stream();
    for (size_t i = 0; i < e->subs.size(); i++) {
        CUDA_TRY(e->d_params[i].ensure(T.params[i].size()));
        CUDA_TRY(cudaMemcpyAsync(e->d_params[i].p, T.params[i].data(), T.params[i].size() * 4, cudaMemcpyHostToDevice, st));
        e->net.sub[i].params = e->d_params[i].p;
        e->net.sub[i].sweep_form = T.sweep_form[i];
        if (T.node_params[i].empty()) { e->net.sub[i].node_params = nullptr; e->net.sub[i].node_pp = 0; continue; }
        CUDA_TRY(e->d_node_params[i].ensure(T.node_params[i].size()));
        CUDA_TRY(cudaMemcpyAsync(e->d_node_params[i].p, T.node_params[i].data(), T.node_params[i].size() * 4,
                                 cudaMemcpyHostToDevice, st));
        e->net.sub[i].node_params = e->d_node_params[i].p;
        e->net.sub[i].node_pp = T.node_pp[i];
    }
    for (size_t p = 0; p < e->projs.size(); p++) {
        HostProj& hp = e->projs[p];
        if (T.cp_pp[p].empty()) { e->net.proj[p].cp_pp = nullptr; continue; }
        if (hp.cp_pp_cap < T.cp_pp[p].size()) {
            if (hp.d_cp_pp) cudaFree(hp.d_cp_pp);
            CUDA_TRY(cudaMalloc(&hp.d_cp_pp, T.cp_pp[p].size() * 4));
            hp.cp_pp_cap = T.cp_pp[p].size();
        }
        CUDA_TRY(cudaMemcpyAsync(hp.d_cp_pp, T.cp_pp[p].data(), T.cp_pp[p].size() * 4, cudaMemcpyHostToDevice, st));
        e->net.proj[p].cp_pp = hp.d_cp_pp;
    }
    CUDA_TRY(cudaMemcpyAsync(e->d_net, &e->net, sizeof(DevNet), cudaMemcpyHostToDevice, st));
    return HB_OK;
}

hb_status reset_bold_device(hb_engine* e) {
    cudaStream_t st = e->stream();
    const int N0 = e->subs[0].nnodes;
    const bool pp = (e->flags & HB_SEM_BOLD_PER_POINT) != 0;
    const size_t lanes = pp ? (size_t)e->B * N0 : (size_t)N0;
    for (auto& bh : e->bold) {
        bh.times.clear();
        bh.n_out = 0;
        bh.out.clear();
        CUDA_TRY(bh.bw.ensure(5 * lanes));
        std::vector<float> init(5 * lanes, 0.0f);
        for (size_t i = 0; i < lanes; i++) { init[lanes + i] = 1.0f; init[2 * lanes + i] = 1.0f; init[3 * lanes + i] = 1.0f; }
        CUDA_TRY(cudaMemcpyAsync(bh.bw.p, init.data(), init.size() * 4, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(bh.acc.ensure((size_t)e->B * N0));
    }
    return HB_OK;
}

// Everything a run needs between its setup (tables, kernel choice, BOLD schedule, launch
// arguments) and its completion (BOLD reductions, flags, bookkeeping).
struct RunPlan {
    int64_t n_steps = 0;
    uint32_t run_flags = 0;
    const float* noise_host = nullptr;
    const float* noise_dev = nullptr;
    bool noise_on_device = false, any_stoch = false, record = false, bold_pp = false, dev_traj = false;
    int64_t noise_rows_per_step = 0, chunk = 0;
    int B = 0, N0 = 0, n_bold_active = 0, stream_npt = 0, fast = -1, pipe = -1, pipe_maxt = 512, single_m = 0;
    int dense_tc = 0, tc_np = 0, tc_kp = 0, tc_npn = 0;  // tensor-core path for undelayed dense coupling
    size_t smem = 0, stream_smem = 0;
    RunArgs a;
    std::vector<std::vector<double>> new_times;
};

hb_status run_setup(hb_engine* e, const RunTables& T, int64_t n_steps, uint32_t run_flags, const float* noise_host,
                    const float* noise_dev, hb_result* res, RunPlan& P) {
    const bool noise_on_device = noise_dev != nullptr;
    cudaStream_t st = e->stream();
    const int B = e->B;
    hb_status s = upload_net(e, T);
    if (s) return s;
    bool any_stoch = false;
    for (auto& sb : e->subs) any_stoch |= is_stochastic(eff_integrator(e, sb.model));
    const bool per_point_noise = (e->flags & HB_SEM_NOISE_PER_POINT) != 0;
    const int64_t noise_rows_per_step = (int64_t)e->noise_row * (per_point_noise ? B : 1);

    // ---- thread layout: `lanes` threads per node share its edge list ----
    {
        int forced = (int)((run_flags >> 12) & 0xf);
        if (run_flags & HB_RUN_EXACT_SUMS) forced = 1;  // one thread per node: its sum in edge order
        std::vector<int> lanes(e->subs.size(), 1);
        for (size_t i = 0; i < e->subs.size(); i++) {
            if (forced) { lanes[i] = 1 << (forced - 1); continue; }
            double deg = 0;
            for (auto& hp : e->projs)
                if (hp.tgt == (int)i && hp.kind == W_SPARSE) deg = std::max(deg, (double)hp.edges.size() / std::max(1, hp.ntgt));
            lanes[i] = deg < 6 ? 1 : deg < 12 ? 2 : deg < 32 ? 4 : 8;
        }
        auto total = [&]() { int t = 0; for (size_t i = 0; i < e->subs.size(); i++) t += (e->subs[i].nm * lanes[i] + 31) / 32 * 32; return t; };
        while (total() > HB_MAX_THREADS) {
            size_t imax = 0;
            for (size_t i = 1; i < lanes.size(); i++) if (lanes[i] > lanes[imax]) imax = i;
            if (lanes[imax] == 1) break;
            lanes[imax] >>= 1;
        }
        if (total() > HB_MAX_THREADS)
            return fail(HB_ERR_UNSUPPORTED, "a sweep point needs %d threads; the point-resident kernel supports %d", total(), HB_MAX_THREADS);
        int off = 0;
        for (size_t i = 0; i < e->subs.size(); i++) {
            DevSub& ds = e->net.sub[i];
            ds.lanes = lanes[i];
            ds.lanes_log2 = 0;
            while ((1 << ds.lanes_log2) < lanes[i]) ds.lanes_log2++;
            ds.thread_off = off;
            off += (e->subs[i].nm * lanes[i] + 31) / 32 * 32;
        }
        e->threads = off;
    }
    // ---- kernel choice: the specialised single-projection form when the network allows it ----
    // ---- tensor-core path for undelayed dense coupling (HB_RUN_DENSE_TC), engine.rs:609-620 ----
    int dense_tc = 0, tc_np = 0, tc_kp = 0, tc_npn = 0;
    if (run_flags & HB_RUN_DENSE_TC) {
        const char* why = nullptr;
        const int km = e->kernel_model;
        if (e->subs.size() != 1 || e->projs.size() != 1) why = "one subnetwork and one projection";
        else {
            const HostProj& hp = e->projs[0];
            const int nm = e->subs[0].nm;
            const int k = hp.cf.kind;
            if (hp.kind != W_SPARSE || hp.src != 0 || hp.tgt != 0) why = "a Dense or CSR projection of the subnetwork onto itself";
            else if (hp.delay != 0 || hp.maxd != 0) why = "no delay";
            else if (!(k == HBC_LINEAR || k == HBC_SIGMOIDAL || k == HBC_SCALED_LINEAR) || hp.diff_mode == 2 || !hp.direct ||
                     hp.ncv != 1 || hp.pc != 1)
                why = "Linear, Sigmoidal or ScaledLinear coupling from and into the first coupling variable";
            else if (!(km == HBM_G2DO || km == HBM_RWW || km == HBM_JR || km == HBM_WC))
                why = "a model with one coupling variable (Generic2dOscillator, ReducedWongWang, JansenRit, WilsonCowan)";
            else if (nm > 112 || hb_dense_tc_tmem_columns(km, nm) > 512)
                why = "at most 112 nodes, with the state and its running sum within tensor memory";
            else if (!e->subs[0].node_params.empty()) why = "one parameter row per point (no node_params)";
            else if ((!e->bold_removed && !e->bold.empty()) || (run_flags & (HB_RUN_TRAJECTORY | HB_RUN_DEVICE_TRAJECTORY)) ||
                     e->cs_out)
                why = "no monitors and no trajectory";
            if (!why) {
                tc_np = (nm + 15) / 16 * 16;
                tc_kp = (nm + 7) / 8 * 8;
                tc_npn = tc_np;
                std::vector<float> w((size_t)nm * nm, 0.0f), tiles((size_t)2 * tc_np * tc_kp);
                for (int i = 0; i < nm; i++)
                    for (int q = hp.rowptr[i]; q < hp.rowptr[i + 1]; q++) w[(size_t)i * nm + (hp.edges[q] & 0xffffu)] = hp.ew[q];
                hb_dense_tc_tiles(w.data(), nm, tc_np, tc_kp, tiles.data());
                CUDA_TRY(e->dtc.ensure(tiles.size()));
                CUDA_TRY(cudaMemcpy(e->dtc.p, tiles.data(), tiles.size() * 4, cudaMemcpyHostToDevice));
                dense_tc = 1;
            }
        }
        if (why) return fail(HB_ERR_UNSUPPORTED, "HB_RUN_DENSE_TC needs %s", why);
    }
    int fast = -1;
    if (e->subs.size() == 1 && e->projs.size() == 1 && e->projs[0].kind == W_SPARSE && !(run_flags & HB_RUN_GENERIC)) {
        const int k = e->projs[0].cf.kind;
        if (k == HBC_LINEAR || k == HBC_SIGMOIDAL || k == HBC_SCALED_LINEAR || k == HBC_DIFFERENCE) fast = 0;  // PRE_ID
        else if (k == HBC_KURAMOTO && e->projs[0].ncv == 1) fast = 1;                                     // PRE_KURA
    }
    e->last_kind = fast >= 0 ? 2 : 1;
    // one warp per point: one subnetwork, one Scalar projection onto itself without delay, no monitors
    int single_m = 0;
    {
        const bool record_run = (run_flags & (HB_RUN_TRAJECTORY | HB_RUN_DEVICE_TRAJECTORY)) != 0;
        const int n_bold_run = e->bold_removed ? 0 : (int)e->bold.size();
        if (e->subs.size() == 1 && e->projs.size() == 1 && e->kernel_model >= 0 && !(run_flags & HB_RUN_GENERIC) &&
            !record_run && n_bold_run == 0 && e->subs[0].nm <= 128 && e->subs[0].node_params.empty()) {
            const HostProj& hp = e->projs[0];
            if ((hp.kind == W_MEAN || hp.kind == W_DIAG) && hp.src == 0 && hp.tgt == 0 && hp.delay == 0)
                single_m = (e->subs[0].nm + 31) / 32;
        }
        if (single_m) e->last_kind = 7;
    }
    // warp-specialised pipeline: one thread per node for the updates plus producer warps, in a
    // 512-thread form or (for more producer lanes or nodes) a 1024-thread form with fewer registers
    int pipe = -1, pipe_maxt = 512;
    if (fast >= 0 && e->dmin >= 15 && !(run_flags & HB_RUN_NO_PIPE) &&
        ((e->subs[0].nm + 31) / 32 * 32 + 64) <= 1024 && !((run_flags >> 12) & 0xf) && !(run_flags & HB_RUN_TWO_PHASE))
        pipe = fast;
    int pipe_lanes = 1;
    if (pipe >= 0) {
        // producer threads: PL lanes per node (a power of two), every node covered, consumers plus
        // producers within the form's thread bound
        const int nm0 = e->subs[0].nm;
        const int n_cons = (nm0 + 31) / 32 * 32;
        auto prod_of = [&](int pl) { return std::max(64, (nm0 * pl + 31) / 32 * 32); };
        const int forced_pl = (run_flags & HB_RUN_EXACT_SUMS) ? 1 : (int)((run_flags >> 20) & 0xf);
        if (forced_pl && ((forced_pl & (forced_pl - 1)) != 0 || forced_pl > 8))
            return fail(HB_ERR_INVALID_STATE, "pipeline producer lanes must be 1, 2, 4 or 8");
        const bool wide = (run_flags & HB_RUN_PIPE_WIDE) || n_cons + 256 > 512 ||
                          (forced_pl && n_cons + prod_of(forced_pl) > 512);
        pipe_maxt = wide ? 1024 : 512;
        const int max_prod = pipe_maxt - n_cons;
        pipe_lanes = forced_pl ? forced_pl : 1;
        if (!forced_pl)
            while (pipe_lanes < 8 && nm0 * pipe_lanes * 2 <= max_prod) pipe_lanes *= 2;
        if (prod_of(pipe_lanes) > max_prod)
            return fail(HB_ERR_UNSUPPORTED, "pipeline: %d nodes x %d producer lanes exceed the thread budget", nm0, pipe_lanes);
        e->threads = n_cons + prod_of(pipe_lanes);
        e->last_kind = 3;
    }
    // ---- placement of the ring and the CSR rows (shared memory when they fit) ----
    const int budget = pipe >= 0 ? (pipe_maxt == 1024 ? hb_pipe_budget_1024(e->kernel_model, pipe) : hb_pipe_budget_512(e->kernel_model, pipe))
                                 : hb_resident_smem_budget(e->kernel_model, fast, e->threads);
    if (budget < 0) return fail(HB_ERR_CUDA, "cannot query the shared-memory limit of the resident kernel");
    const size_t smem_cap = (size_t)budget - 64;
    size_t part_bytes = (size_t)2 * std::max(e->n_mean, 1) * 32 * 4 * 4;
    if (pipe >= 0) {
        // gx and noise double buffers: [2][8][nm][channels] + [2][8][nm*nvar]
        const int pch = (pipe == 1) ? 2 : e->subs[0].ncvar;
        part_bytes = (size_t)2 * 8 * e->subs[0].nm * (pch + (any_stoch ? e->subs[0].nvar : 0)) * 4 +
                     (size_t)(e->subs[0].nm + 1) * 4 + 48;
    }
    // ring length of this run: the pipeline's producers run at most one block ahead of the consumers'
    // writes, so slot reuse needs only more slots than the longest delay; the other kernels keep the
    // engine's ring (longest delay + their barrier interval)
    const int R_run = pipe >= 0 ? std::max(e->H, 1) + 1 : e->R;
    e->net.R = R_run;
    // (the pipeline's ring in shared memory carries 8 mirror slots, one block of steps, after its R slots)
    const size_t ring_bytes = (size_t)(R_run + (pipe >= 0 ? 8 : 0)) * e->cols * 4;
    size_t edges = 0;
    for (auto& hp : e->projs) if (hp.kind == W_SPARSE) edges += hp.edges.size();
    const size_t edge_bytes = ((edges * 8) + 15) & ~(size_t)15;
    int ring_in_smem = 0, edges_in_smem = 0;
    bool force_global = (run_flags & HB_RUN_GLOBAL_RING) != 0;
    if (!force_global && ring_bytes + 16 + edge_bytes + part_bytes <= smem_cap) { ring_in_smem = 1; edges_in_smem = 1; }
    else if (!force_global && ring_bytes + 16 + part_bytes <= smem_cap) { ring_in_smem = 1; }
    else if (edge_bytes + part_bytes <= smem_cap) { edges_in_smem = 1; }
    size_t smem = (ring_in_smem ? ((ring_bytes + 15) & ~(size_t)15) : 0) + (edges_in_smem ? edge_bytes : 0) + part_bytes + 16;
    // ---- streamed-history pipeline: per-edge delays whose history does not fit shared memory ----
    int stream_npt = 0, stream_pl = 1, stream_rp = 0, stream_noise_smem = 0, stream_edges = 0, stream_cluster = 1;
    int stream_wgather = 0, stream_bulk = 0;
    size_t stream_smem = 0;
    if (fast >= 0 && e->projs[0].dmode == HBD_EDGE && e->dmin >= 2 * HB_STREAM_K - 1 && !(run_flags & HB_RUN_NO_STREAM) &&
        (!ring_in_smem || (run_flags & HB_RUN_STREAM)) && !((run_flags >> 12) & 0xf) && !(run_flags & HB_RUN_TWO_PHASE) &&
        !(run_flags & HB_RUN_GLOBAL_RING)) {
        const int nm_all = e->subs[0].nm, nvar0 = e->subs[0].nvar;
        const int pch = (fast == 1) ? 2 : e->subs[0].ncvar;
        // consumer threads per CTA: one node per thread (512 threads) for up to 96 nodes, else two (1024
        // threads, at least 256 producers); four (768 threads, two edge windows in flight per producer) on
        // request
        const int want = (int)((run_flags >> 24) & 0x7);
        auto plan_threads = [&](int nmx, int& np_, int& nt_) {
            auto fits = [&](int k, int nt) { return ((nmx + k - 1) / k + 31) / 32 * 32 + (nt == 512 ? 128 : 256) <= nt; };
            np_ = 0;
            nt_ = 0;
            if (want == 1 || (want == 0 && nmx <= 96)) { if (fits(1, 512)) { np_ = 1; nt_ = 512; } }
            else if (want == 4) { if (fits(4, 768)) { np_ = 4; nt_ = 768; } }
            else if (fits(2, 1024)) { np_ = 2; nt_ = 1024; }
        };
        // CTAs per point: a thread-block cluster splitting the point's nodes (HB_RUN_STREAM_CLUSTER), so
        // that fewer points are in flight and their histories stay in L2
        {
            static const int code_to_c[8] = {0, 1, 2, 4, 8, 3, 5, 6};
            const int v = (int)((run_flags >> 4) & 0x7);
            if (v == 0) {
                // engine's choice among 1..6 and 8 CTAs per point (at least 64 nodes per CTA): the size whose
                // resident clusters (one point each, as the device's cluster occupancy reports them) keep the
                // histories in flight within about 100 MB of the 129 MB L2, then the most SMs busy
                int dev = 0, sms = 152;
                if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                const int rp = (e->projs[0].maxd + 2 * HB_STREAM_K + 2 + 7) / 8 * 8;
                const double hist = (double)nm_all * (rp + 2 * HB_STREAM_K) * pch * 4;
                static const int cand[7] = {1, 2, 3, 4, 5, 6, 8};
                double best = -1.0;
                bool best_fit = false;
                stream_cluster = 1;
                for (int c : cand) {
                    if (c > 1 && nm_all / c < 64) continue;
                    const int nmx = (nm_all + c - 1) / c;
                    int np_ = 0, nt_ = 0;
                    plan_threads(nmx, np_, nt_);
                    if (!np_) continue;
                    const size_t smem_est = (size_t)2 * HB_STREAM_K * nmx * pch * 4 + (size_t)nmx * 16 + 1024;
                    const int cap = c == 1 ? sms
                                  : np_ == 1 ? hb_stream_clusters_1(e->kernel_model, fast, c, nt_, smem_est)
                                  : np_ == 2 ? hb_stream_clusters_2(e->kernel_model, fast, c, nt_, smem_est)
                                             : hb_stream_clusters_4(e->kernel_model, fast, c, nt_, smem_est);
                    if (cap <= 0) continue;
                    const double inflight = std::min<double>(B, cap);
                    const bool fit = inflight * hist <= 100e6;
                    const double score = inflight * c;  // SMs busy
                    if (best < 0 || (fit && !best_fit) || (fit == best_fit && score > best)) {
                        best = score;
                        best_fit = fit;
                        stream_cluster = c;
                    }
                }
            } else stream_cluster = code_to_c[v];
            if (stream_cluster > 8 || stream_cluster > nm_all)
                return fail(HB_ERR_INVALID_STATE, "HB_RUN_STREAM_CLUSTER: 1 to 6 or 8 CTAs per point, at most one per node");
        }
        const int SC = stream_cluster;
        const int nm0 = (nm_all + SC - 1) / SC;  // nodes of the largest slice
        size_t slice_edges = 0;
        for (int r = 0; r < SC; r++) {
            const int a0 = (int)(((long long)nm_all * r) / SC), a1 = (int)(((long long)nm_all * (r + 1)) / SC);
            slice_edges = std::max(slice_edges, (size_t)(e->projs[0].rowptr[a1] - e->projs[0].rowptr[a0]));
        }
        int npt = 0, threads = 0;
        plan_threads(nm0, npt, threads);
        const int sbudget = npt == 1 ? hb_stream_budget_1(e->kernel_model, fast)
                          : npt == 2 ? hb_stream_budget_2(e->kernel_model, fast)
                          : npt == 4 ? hb_stream_budget_4(e->kernel_model, fast) : -1;
        if (npt && sbudget > 0) {
            const size_t cap = (size_t)sbudget - 64;
            const size_t gx_b = (size_t)2 * HB_STREAM_K * nm0 * pch * 4;
            const size_t nz_b = any_stoch ? (size_t)2 * HB_STREAM_K * nm0 * nvar0 * 4 : 0;
            const size_t rp_b = ((size_t)(nm0 + 1) * 4 + 15) & ~(size_t)15;
            const size_t ed_b = slice_edges * 8;
            const size_t pr_b = stream_prm_bytes(e->kernel_model, nm0, npt) + (size_t)nm0 * 4 + 16;  // + producer order
            if (gx_b + rp_b + pr_b + 16 <= cap) {
                stream_npt = npt;
                stream_noise_smem = (nz_b > 0 && gx_b + nz_b + rp_b + pr_b + 16 <= cap) ? 1 : 0;
                size_t used = gx_b + (stream_noise_smem ? nz_b : 0) + rp_b + pr_b + 16;
                if (used + ed_b + 16 <= cap) { stream_edges = (int)slice_edges; used += ed_b + 16; }
                stream_smem = used;
                const int n_cons = ((nm0 + npt - 1) / npt + 31) / 32 * 32;
                const int n_prod = threads - n_cons;
                const int forced_pl = (int)((run_flags >> 20) & 0xf);
                if (forced_pl && ((forced_pl & (forced_pl - 1)) != 0 || forced_pl > 8))
                    return fail(HB_ERR_INVALID_STATE, "producer lanes must be 1, 2, 4 or 8");
                if (run_flags & HB_RUN_EXACT_SUMS) stream_pl = 1;
                else if (forced_pl) stream_pl = forced_pl;
                else
                    while (stream_pl < 8 && nm0 * stream_pl * 2 <= n_prod) stream_pl *= 2;
                e->threads = threads;
                // warp-cooperative gathers (unless the reference's summation order or a producer lane count
                // is asked for) when the slice's edge lists sit in shared memory and the nodes' rows fill most
                // of the warp's 32-edge chunks (a mean in-degree of at least 24). With the edge lists in
                // global memory each chunk's descriptor load would precede its window loads on the critical
                // path, and one thread per window keeps more loads in flight there.
                if (!(run_flags & HB_RUN_EXACT_SUMS) && !((run_flags >> 20) & 0xf) && stream_edges > 0 &&
                    e->projs[0].edges.size() >= (size_t)24 * nm_all)
                    stream_wgather = 1;
                // HB_RUN_STREAM_BULK: the warp gather's windows staged by the bulk-copy engine, 32 slots per
                // producer warp (80 bytes for two channels, 48 for one) and one mbarrier per warp
                if (run_flags & HB_RUN_STREAM_BULK) {
                    if (!stream_wgather)
                        return fail(HB_ERR_UNSUPPORTED, "HB_RUN_STREAM_BULK needs the warp-cooperative gather (edge lists in shared "
                                    "memory, mean in-degree >= 24, no exact sums or producer lane count)");
                    const size_t bulk_b = (size_t)(n_prod / 32) * (32 * (pch == 2 ? 80 : 48) + 8) + 16;
                    if (stream_smem + bulk_b > cap)
                        return fail(HB_ERR_UNSUPPORTED, "HB_RUN_STREAM_BULK: the staging area does not fit shared memory");
                    stream_smem += bulk_b;
                    stream_bulk = 1;
                }
                stream_rp = (e->projs[0].maxd + 2 * HB_STREAM_K + 2 + 7) / 8 * 8;
                const size_t words = (size_t)B * nm_all * (stream_rp + 2 * HB_STREAM_K) * pch;
                CUDA_TRY(e->sring.ensure(words));
                e->last_kind = 4;
            }
        }
    }
    {
        const int layout = dense_tc ? 3 : stream_npt ? 1 : 0;
        if (e->step > 0 && (layout != e->hist_layout || (layout == 1 && stream_rp != e->hist_rp) ||
                            (layout == 0 && R_run != e->hist_R)))
            return fail(HB_ERR_UNSUPPORTED, "this run would change the history layout of a started simulation; reset the engine first");
        e->hist_layout = layout;
        e->hist_rp = stream_rp;
        e->hist_R = R_run;
    }
    {
        size_t off = 0;
        for (size_t p = 0; p < e->projs.size(); p++) {
            if (e->projs[p].kind == W_SPARSE && edges_in_smem) { e->net.proj[p].smem_edges = (int)off; off += e->projs[p].edges.size(); }
            else e->net.proj[p].smem_edges = -1;
            e->net.proj[p].porder = nullptr;
        }
        // producer order of the pipeline and streamed-history kernels: each node slice's nodes by
        // decreasing in-degree (a warp's lanes then walk similar numbers of edges; every node's own sum
        // is unchanged)
        if (pipe >= 0 || stream_npt) {
            const HostProj& hp = e->projs[0];
            const int nmo = e->subs[0].nm, SC = stream_npt ? stream_cluster : 1;
            std::vector<int> order(nmo);
            for (int r = 0; r < SC; r++) {
                const int a0 = (int)(((long long)nmo * r) / SC), a1 = (int)(((long long)nmo * (r + 1)) / SC);
                for (int i = a0; i < a1; i++) order[i] = i - a0;
                std::stable_sort(order.begin() + a0, order.begin() + a1, [&](int x, int y) {
                    return hp.rowptr[a0 + x + 1] - hp.rowptr[a0 + x] > hp.rowptr[a0 + y + 1] - hp.rowptr[a0 + y];
                });
            }
            CUDA_TRY(e->porder.ensure(nmo));
            CUDA_TRY(cudaMemcpyAsync(e->porder.p, order.data(), nmo * sizeof(int), cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaStreamSynchronize(st));  // `order` is released at scope end
            e->net.proj[0].porder = e->porder.p;
        }
        CUDA_TRY(cudaMemcpyAsync(e->d_net, &e->net, sizeof(DevNet), cudaMemcpyHostToDevice, st));
    }

    // ---- BOLD schedule of this run ----
    const int n_bold_active = e->bold_removed ? 0 : (int)e->bold.size();
    const bool bold_pp = (e->flags & HB_SEM_BOLD_PER_POINT) != 0;
    const int N0 = e->subs[0].nnodes;
    DevBold db;
    memset(&db, 0, sizeof db);
    db.n = n_bold_active;
    db.per_point = bold_pp ? 1 : 0;
    db.n0 = N0;
    std::vector<std::vector<double>> new_times(n_bold_active);
    for (int m = 0; m < n_bold_active; m++) {
        BoldHost& bh = e->bold[m];
        std::vector<BoldEmit> emit;
        int n_full, partial;
        int64_t n_new = bold_schedule(e, bh, n_steps, emit, n_full, partial, new_times[m]);
        db.period[m] = bh.period;
        db.n_full[m] = n_full;
        db.partial[m] = partial;
        db.dt_full[m] = (float)((e->dt_ms * (double)bh.period) / 1000.0);
        db.dt_part[m] = (float)((e->dt_ms * (double)partial) / 1000.0);
        db.n_emit[m] = (int)emit.size();
        CUDA_TRY(bh.emit.ensure(emit.size()));
        if (!emit.empty()) CUDA_TRY(cudaMemcpyAsync(bh.emit.p, emit.data(), emit.size() * sizeof(BoldEmit), cudaMemcpyHostToDevice, st));
        db.emit[m] = bh.emit.p;
        db.n_out_run[m] = (int)n_new;
        CUDA_TRY(bh.out_run.ensure((size_t)std::max<int64_t>(n_new, 1) * N0 * (bold_pp ? B : 1)));
        db.out[m] = bh.out_run.p;
        db.bw[m] = bh.bw.p;
        db.acc[m] = bh.acc.p;
        if (!bold_pp) {
            int n_win = n_full + (partial > 0 ? 1 : 0);
            CUDA_TRY(bh.win.ensure((size_t)std::max(n_win, 1) * B * N0));
            db.win[m] = bh.win.p;
        }
        CUDA_TRY(cudaStreamSynchronize(st));  // the emit vector is released at scope end
    }

    // ---- chunking: one launch unless a trajectory or per-point noise must be streamed ----
    const bool record = (run_flags & HB_RUN_TRAJECTORY) != 0;
    int64_t chunk = n_steps;
    const size_t traj_step_bytes = (size_t)B * e->state_len * 4;
    if (record && !(run_flags & HB_RUN_DEVICE_TRAJECTORY))
        chunk = std::max<int64_t>(1, std::min<int64_t>(chunk, (int64_t)((512ull << 20) / std::max<size_t>(traj_step_bytes, 1))));
    if (any_stoch && !noise_on_device) {
        const size_t nb = (size_t)noise_rows_per_step * 4;
        chunk = std::max<int64_t>(1, std::min<int64_t>(chunk, (int64_t)((2048ull << 20) / std::max<size_t>(nb, 1))));
    }
    chunk = std::min<int64_t>(chunk, (int64_t)1 << 30);
    const bool dev_traj = (run_flags & HB_RUN_DEVICE_TRAJECTORY) != 0;
    if (dev_traj) {
        const size_t need = (size_t)n_steps * traj_step_bytes;
        if (e->dtraj.n * 4 < need) {
            e->dtraj.release();
            size_t free_b = 0, total_b = 0;
            CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
            if (need + (256ull << 20) > free_b)
                return fail(HB_ERR_UNSUPPORTED, "device trajectory needs %.2f GB, %.2f GB free", need / 1e9, free_b / 1e9);
            CUDA_TRY(e->dtraj.ensure(need / 4));
        }
    }
    e->dtraj_steps = 0;
    if (record && res) {
        if (!dev_traj) CUDA_TRY(e->traj.ensure((size_t)chunk * B * e->state_len));
        res->traj.assign(e->subs.size(), std::vector<float>());
        for (size_t i = 0; i < e->subs.size(); i++) res->traj[i].resize((size_t)n_steps * B * e->subs[i].nm * e->subs[i].nvar);
    }
    if (any_stoch && !noise_on_device) CUDA_TRY(e->noise.ensure((size_t)chunk * noise_rows_per_step));
    CUDA_TRY(e->flags_buf.ensure(2));
    CUDA_TRY(cudaMemsetAsync(e->flags_buf.p, 0, 2 * sizeof(int), st));

    RunArgs a;
    memset(&a, 0, sizeof a);
    a.run_s0 = e->step;
    a.run_steps = n_steps;
    a.state = e->state.p;
    a.tavg = e->tavg.p;
    a.ring = e->ring.p;
    a.noise_per_point = per_point_noise ? 1 : 0;
    a.ring_in_smem = ring_in_smem;
    a.sync_every = fast >= 0 ? e->sync_every : 1;
    a.two_phase = (run_flags & HB_RUN_TWO_PHASE) ? 1 : 0;
    a.pipe_lanes = stream_npt ? stream_pl : pipe_lanes;
    a.smem_edges = stream_npt ? stream_edges : (edges_in_smem ? (int)edges : 0);
    a.stream_rp = stream_rp;
    a.stream_noise_smem = stream_noise_smem;
    a.stream_prefetch = (run_flags & HB_RUN_STREAM_PREFETCH) ? 2 : 0;
    a.stream_cluster = stream_npt ? stream_cluster : 1;
    if (stream_npt) { a.ring = e->sring.p; a.ring_in_smem = 0; }
    a.flags = e->flags_buf.p;
    a.check_finite = (run_flags & HB_RUN_CHECK_FINITE) ? 1 : 0;
    a.test_unset_wait = (run_flags & HB_RUN_TEST_UNSET_WAIT) ? 1 : 0;
    a.exact_sums = (run_flags & HB_RUN_EXACT_SUMS) ? 1 : 0;
    a.stream_wgather = stream_npt ? stream_wgather : 0;
    a.stream_bulk = stream_npt ? stream_bulk : 0;
    a.bold = db;

    P.n_steps = n_steps;
    P.run_flags = run_flags;
    P.noise_host = noise_host;
    P.noise_dev = noise_dev;
    P.noise_on_device = noise_on_device;
    P.any_stoch = any_stoch;
    P.record = record;
    P.dev_traj = dev_traj;
    P.bold_pp = bold_pp;
    P.noise_rows_per_step = noise_rows_per_step;
    P.chunk = chunk;
    P.B = B;
    P.N0 = N0;
    P.n_bold_active = n_bold_active;
    P.stream_npt = stream_npt;
    P.fast = fast;
    P.pipe = pipe;
    P.pipe_maxt = pipe_maxt;
    P.single_m = single_m;
    P.dense_tc = dense_tc;
    P.tc_np = tc_np;
    P.tc_kp = tc_kp;
    P.tc_npn = tc_npn;
    if (dense_tc) e->last_kind = 8;
    P.smem = smem;
    P.stream_smem = stream_smem;
    P.a = a;
    P.new_times.swap(new_times);
    return HB_OK;
}

// the launches of a run: one, or one per chunk when a trajectory or host noise is streamed
hb_status run_launch(hb_engine* e, RunPlan& P, hb_result* res) {
    cudaStream_t st = e->stream();
    const int B = P.B;
    const int64_t n_steps = P.n_steps, chunk = P.chunk, noise_rows_per_step = P.noise_rows_per_step;
    const bool any_stoch = P.any_stoch, noise_on_device = P.noise_on_device, record = P.record, dev_traj = P.dev_traj;
    const float* noise_dev = P.noise_dev;
    const float* noise_host = P.noise_host;
    const int stream_npt = P.stream_npt, fast = P.fast, pipe = P.pipe;
    const size_t smem = P.smem, stream_smem = P.stream_smem;
    RunArgs& a = P.a;
    std::vector<float> traj_host;
    e->last_launches = 0;
    float kernel_ms_total = 0.0f;
    for (int64_t c0 = 0; c0 < n_steps; c0 += chunk) {
        const int n = (int)std::min<int64_t>(chunk, n_steps - c0);
        a.s0 = e->step + c0;
        a.n_steps = n;
        a.load_ring = (a.s0 > 0) ? 1 : 0;
        a.store_ring = 1;
        if (any_stoch) {
            if (noise_on_device) a.noise = noise_dev + (size_t)c0 * noise_rows_per_step;
            else {
                CUDA_TRY(cudaMemcpyAsync(e->noise.p, noise_host + (size_t)c0 * noise_rows_per_step,
                                         (size_t)n * noise_rows_per_step * 4, cudaMemcpyHostToDevice, st));
                a.noise = e->noise.p;
            }
        }
        float* traj_dst = dev_traj ? e->dtraj.p + (size_t)c0 * B * e->state_len : e->traj.p;
        a.traj = (record || dev_traj) ? traj_dst : nullptr;
        a.gx_out = e->cs_out ? e->cs_out + (size_t)c0 * B * e->subs[0].nm * 2 : nullptr;
        CUDA_TRY(cudaEventRecord(e->ev0, st));
        if (P.dense_tc) CUDA_TRY(hb_launch_dense_tc(e->kernel_model, e->d_net, a, B, e->dtc.p, P.tc_np, P.tc_kp, P.tc_npn, st));
        else if (P.single_m) CUDA_TRY(hb_launch_single(e->kernel_model, P.single_m, e->d_net, a, B, st));
        else if (stream_npt == 1) CUDA_TRY(hb_launch_stream_1(e->kernel_model, fast, e->d_net, a, B, e->threads, stream_smem, st));
        else if (stream_npt == 2) CUDA_TRY(hb_launch_stream_2(e->kernel_model, fast, e->d_net, a, B, e->threads, stream_smem, st));
        else if (stream_npt == 4) CUDA_TRY(hb_launch_stream_4(e->kernel_model, fast, e->d_net, a, B, e->threads, stream_smem, st));
        else if (pipe >= 0 && P.pipe_maxt == 1024) CUDA_TRY(hb_launch_pipe_1024(e->kernel_model, pipe, e->d_net, a, B, e->threads, smem, st));
        else if (pipe >= 0) CUDA_TRY(hb_launch_pipe_512(e->kernel_model, pipe, e->d_net, a, B, e->threads, smem, st));
        else CUDA_TRY(hb_launch_resident(e->kernel_model, fast, e->d_net, a, B, e->threads, smem, st));
        CUDA_TRY(cudaEventRecord(e->ev1, st));
        e->last_launches++;
        if (record) {
            traj_host.resize((size_t)n * B * e->state_len);
            CUDA_TRY(cudaMemcpyAsync(traj_host.data(), traj_dst, traj_host.size() * 4, cudaMemcpyDeviceToHost, st));
        }
        CUDA_TRY(cudaEventSynchronize(e->ev1));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
        kernel_ms_total += ms;
        if (record) {
            CUDA_TRY(cudaStreamSynchronize(st));
            // [step][B][state_len] -> per subnetwork [step][B][nm*nvar]
            for (int it = 0; it < n; it++)
                for (int b = 0; b < B; b++)
                    for (size_t i = 0; i < e->subs.size(); i++) {
                        const int per = e->subs[i].nm * e->subs[i].nvar;
                        const float* src = traj_host.data() + ((size_t)it * B + b) * e->state_len + e->net.sub[i].state_off;
                        float* dst = res->traj[i].data() + (((size_t)(c0 + it)) * B + b) * per;
                        memcpy(dst, src, per * 4);
                    }
        }
    }
    e->last_ms = kernel_ms_total;
    e->dtraj_steps = dev_traj ? n_steps : 0;
    return HB_OK;
}

// completion of a run after its launches: batch-mean BOLD, flags, step counter, BOLD outputs
hb_status run_finish(hb_engine* e, RunPlan& P, hb_result* res, bool device_part = true) {
    cudaStream_t st = e->stream();
    const int B = P.B, N0 = P.N0, n_bold_active = P.n_bold_active;
    const bool bold_pp = P.bold_pp;
    const int64_t n_steps = P.n_steps;
    const DevBold& db = P.a.bold;
    const RunArgs& a = P.a;
    std::vector<std::vector<double>>& new_times = P.new_times;

    // ---- batch-mean BOLD: reduce windows over sweep points, then the BW ODE ----
    for (int m = 0; m < n_bold_active && !bold_pp && device_part; m++) {
        int n_win = db.n_full[m] + (db.partial[m] > 0 ? 1 : 0);
        CUDA_TRY(e->means.ensure((size_t)std::max(n_win, 1) * N0));
        CUDA_TRY(hb_launch_bold_batch_mean(db, m, n_win, B, e->means.p, st));
    }
    int flags_h[2] = {0, 0};
    CUDA_TRY(cudaMemcpyAsync(flags_h, e->flags_buf.p, sizeof flags_h, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    e->step += n_steps;
    // BOLD bookkeeping and outputs
    for (int m = 0; m < n_bold_active; m++) {
        BoldHost& bh = e->bold[m];
        bh.times.insert(bh.times.end(), new_times[m].begin(), new_times[m].end());
        int64_t n_new = db.n_out_run[m];
        if (res && n_new > 0) {
            std::vector<float> tmp((size_t)n_new * N0 * (bold_pp ? B : 1));
            CUDA_TRY(cudaMemcpy(tmp.data(), bh.out_run.p, tmp.size() * 4, cudaMemcpyDeviceToHost));
            if (!bold_pp) bh.out.insert(bh.out.end(), tmp.begin(), tmp.end());
            else {
                std::vector<float> merged((size_t)B * (bh.n_out + n_new) * N0);
                for (int b = 0; b < B; b++) {
                    if (bh.n_out) memcpy(&merged[(size_t)b * (bh.n_out + n_new) * N0], &bh.out[(size_t)b * bh.n_out * N0], (size_t)bh.n_out * N0 * 4);
                    memcpy(&merged[((size_t)b * (bh.n_out + n_new) + bh.n_out) * N0], &tmp[(size_t)b * n_new * N0], (size_t)n_new * N0 * 4);
                }
                bh.out.swap(merged);
            }
        }
        bh.n_out += n_new;
    }
    if (flags_h[1] & 4) return fail(HB_ERR_TIMEOUT, "a bounded device-side wait on a bulk copy gave up");
    if (a.check_finite && flags_h[0]) return fail(HB_ERR_NONFINITE, "a state variable became NaN or Inf");
    return HB_OK;
}

// the simulation of one run; noise is a host pointer (copied per launch) or a device pointer
hb_status run_device(hb_engine* e, const RunTables& T, int64_t n_steps, uint32_t run_flags, const float* noise_host,
                     const float* noise_dev, hb_result* res) {
    RunPlan P;
    hb_status s = run_setup(e, T, n_steps, run_flags, noise_host, noise_dev, res, P);
    if (s) return s;
    s = run_launch(e, P, res);
    if (s) return s;
    return run_finish(e, P, res);
}

hb_status collect(hb_engine* e, int64_t n_steps, hb_result* r) {
    const int B = e->B;
    std::vector<float> st((size_t)B * e->state_len), ta((size_t)B * e->state_len);
    CUDA_TRY(cudaMemcpyAsync(st.data(), e->state.p, st.size() * 4, cudaMemcpyDeviceToHost, e->stream()));
    CUDA_TRY(cudaMemcpyAsync(ta.data(), e->tavg.p, ta.size() * 4, cudaMemcpyDeviceToHost, e->stream()));
    CUDA_TRY(cudaStreamSynchronize(e->stream()));
    const float inv = 1.0f / (float)n_steps;  // engine.rs:514
    r->tavg.assign(e->subs.size(), {});
    r->fin.assign(e->subs.size(), {});
    for (size_t i = 0; i < e->subs.size(); i++) {
        const int per = e->subs[i].nm * e->subs[i].nvar;
        r->tavg[i].resize((size_t)B * per);
        r->fin[i].resize((size_t)B * per);
        for (int b = 0; b < B; b++)
            for (int k = 0; k < per; k++) {
                size_t src = (size_t)b * e->state_len + e->net.sub[i].state_off + k;
                r->tavg[i][(size_t)b * per + k] = ta[src] * inv;
                r->fin[i][(size_t)b * per + k] = st[src];
            }
    }
    const int n_bold_active = e->bold_removed ? 0 : (int)e->bold.size();
    r->n_bold = n_bold_active;
    r->bold.assign(n_bold_active, {});
    for (int m = 0; m < n_bold_active; m++) r->bold[m] = e->bold[m].out;
    r->n_sweep = B;
    return HB_OK;
}

hb_status validate_noise(hb_engine* e, const float* noise, int64_t noise_len, int64_t n_steps) {
    bool any = false;
    for (auto& s : e->subs) any |= is_stochastic(eff_integrator(e, s.model));
    if (!any) return HB_OK;
    int64_t need = (int64_t)e->noise_row * ((e->flags & HB_SEM_NOISE_PER_POINT) ? e->B : 1) * n_steps;
    if (!noise || noise_len < need)
        return fail(HB_ERR_INVALID_STATE, "noise array too short: %lld < %lld", (long long)noise_len, (long long)need);
    for (size_t i = 0; i < e->subs.size(); i++)
        if (e->subs[i].nvar > (int)e->nsig.size())
            return fail(HB_ERR_INVALID_CONFIG, "nsig has %d entries, subnetwork %d has nvar %d", (int)e->nsig.size(), (int)i, e->subs[i].nvar);
    return HB_OK;
}

hb_status reset_state(hb_engine* e) {
    CUDA_TRY(cudaMemcpyAsync(e->state.p, e->x0.p, (size_t)e->B * e->state_len * 4, cudaMemcpyDeviceToDevice, e->stream()));
    e->step = 0;
    return HB_OK;
}

}  // namespace

// error message setter for the other translation units of the library (not exported)
__attribute__((visibility("hidden"))) void hb_internal_set_error(const char* msg) { g_err = msg ? msg : ""; }

// ======================================================================================
// C ABI
// ======================================================================================
extern "C" {

int32_t hb_abi_version(void) { return HB_ABI_VERSION; }
const char* hb_last_error(void) { return g_err.c_str(); }

hb_status hb_model_info(const char* model, int32_t* nvar, int32_t* ncvar, int32_t* n_params) {
    if (!nvar || !ncvar || !n_params) return fail(HB_ERR_INVALID_STATE, "NULL output pointer");
    int m = model_id(model);
    if (m >= 0) { *nvar = k_models[m].nvar; *ncvar = k_models[m].ncvar; *n_params = k_models[m].nparams; return HB_OK; }
    for (int i = 0; i < 22; i++)
        if (model && !strcmp(model, k_other_models[i])) { *nvar = k_other_nvar[i]; *ncvar = k_other_ncvar[i]; *n_params = k_other_np[i]; return HB_OK; }
    return fail(HB_ERR_INVALID_CONFIG, "Unknown model '%s'. Known models: %s", model ? model : "(null)",
                known_models().c_str());
}

hb_status hb_engine_create(const hb_sim_desc* d, int32_t n_sweep, hb_engine** out) {
    if (!out) return fail(HB_ERR_INVALID_STATE, "out is NULL");
    *out = nullptr;
    if (!d) return fail(HB_ERR_INVALID_CONFIG, "descriptor is NULL");
    if (n_sweep < 1) return fail(HB_ERR_INVALID_CONFIG, "n_sweep must be >= 1");
    if (d->n_subnets < 1) return fail(HB_ERR_INVALID_CONFIG, "At least one subnetwork required");
    if (d->n_subnets > HB_MAX_SUB) return fail(HB_ERR_UNSUPPORTED, "at most %d subnetworks are supported", HB_MAX_SUB);
    if (d->n_projections > HB_MAX_PROJ) return fail(HB_ERR_UNSUPPORTED, "at most %d projections are supported", HB_MAX_PROJ);
    if (d->n_bold > HB_MAX_BOLD) return fail(HB_ERR_UNSUPPORTED, "at most %d BOLD monitors are supported", HB_MAX_BOLD);
    if (!(d->dt > 0.0)) return fail(HB_ERR_INVALID_CONFIG, "dt must be positive");
    if (d->integrator < 0 || d->integrator > 5) return fail(HB_ERR_INVALID_CONFIG, "unknown integrator kind: %d", d->integrator);
    const bool ring = (d->flags & HB_SEM_DELAY_RING) != 0;

    hb_engine* e = new hb_engine();
    auto bail = [&](hb_status s) { hb_engine_destroy(e); return s; };
    e->B = n_sweep;
    e->dt_ms = d->dt;
    e->integrator = d->integrator;
    e->flags = d->flags;
    e->nsig.assign(d->nsig, d->nsig + std::max(0, d->n_nsig));
    memset(&e->net, 0, sizeof e->net);

    // ---- subnetworks (engine.rs:153-247) ----
    int thread_off = 0, col_off = 0, state_off = 0;
    for (int i = 0; i < d->n_subnets; i++) {
        const hb_subnet_desc& sd = d->subnets[i];
        HostSub s;
        s.model = model_id(sd.model);
        if (s.model < 0) {
            if (is_other_model(sd.model))
                return bail(fail(HB_ERR_UNSUPPORTED, "model '%s' is not batch-native in the reference (per-point fallback); "
                                 "this engine implements the six batch-native models", sd.model));
            return bail(fail(HB_ERR_INVALID_CONFIG, "Unknown model '%s' in subnetwork %d. Known models: %s",
                             sd.model ? sd.model : "(null)", i, known_models().c_str()));
        }
        // messages of SimConfig::validate (config.rs:305-309) where it checks the same thing
        if (sd.nmodes < 1) return bail(fail(HB_ERR_INVALID_CONFIG, "Subnetwork %d: nmodes must be >= 1", i));
        if (sd.nnodes < 1) return bail(fail(HB_ERR_INVALID_CONFIG, "Subnetwork %d: nnodes must be >= 1", i));
        s.nnodes = sd.nnodes; s.nmodes = sd.nmodes; s.nm = sd.nnodes * sd.nmodes;
        s.nvar = k_models[s.model].nvar; s.ncvar = k_models[s.model].ncvar;
        if (sd.n_params < k_models[s.model].nparams || sd.n_params > 24)
            return bail(fail(HB_ERR_INVALID_CONFIG, "Subnetwork %d: model '%s' expects %d params, got %d", i, sd.model,
                             k_models[s.model].nparams, sd.n_params));
        s.nparams = sd.n_params;
        s.params.assign(sd.params, sd.params + sd.n_params);
        if (sd.n_initial_state != (int64_t)s.nm * s.nvar)
            return bail(fail(HB_ERR_INVALID_CONFIG, "Subnetwork %d: initial_state has %lld values, expected %d (nvar=%d * nnodes=%d * nmodes=%d)",
                             i, (long long)sd.n_initial_state, s.nm * s.nvar, s.nvar, s.nnodes, s.nmodes));
        s.x0.assign(sd.initial_state, sd.initial_state + s.nm * s.nvar);
        if (sd.n_node_params > 0) {
            const int64_t per = (int64_t)s.nm * sd.n_params;
            if (!sd.node_params || (sd.n_node_params != per && sd.n_node_params != per * n_sweep))
                return bail(fail(HB_ERR_INVALID_CONFIG, "Subnetwork %d: node_params has %lld values, expected %lld "
                                 "(nnodes*nmodes * n_params) or %lld (n_sweep * nnodes*nmodes * n_params)", i,
                                 (long long)sd.n_node_params, (long long)per, (long long)(per * n_sweep)));
            s.node_params.assign(sd.node_params, sd.node_params + sd.n_node_params);
            s.node_pp = sd.n_node_params != per || n_sweep == 1;
        }
        if (ring && s.nmodes != 1) return bail(fail(HB_ERR_UNSUPPORTED, "ring-buffer delay semantics need nmodes == 1"));
        if (s.nm > 65535) return bail(fail(HB_ERR_UNSUPPORTED, "subnetwork %d has %d nodes; at most 65535 are supported", i, s.nm));
        DevSub& ds = e->net.sub[i];
        ds.model = s.model; ds.nm = s.nm; ds.nvar = s.nvar; ds.ncvar = s.ncvar;
        ds.thread_off = thread_off; ds.col_off = col_off; ds.state_off = state_off; ds.noise_off = state_off;
        ds.lanes = 1; ds.lanes_log2 = 0;
        thread_off += (s.nm + 31) / 32 * 32;
        col_off += s.nm * s.ncvar;
        state_off += s.nm * s.nvar;
        e->subs.push_back(s);
    }
    e->threads = thread_off;
    e->cols = col_off;
    e->state_len = state_off;
    e->noise_row = state_off;
    if (e->threads > HB_MAX_THREADS)
        return bail(fail(HB_ERR_UNSUPPORTED, "a sweep point has %d node threads; the point-resident kernel supports %d", e->threads, HB_MAX_THREADS));

    // ---- horizon: engine.rs:253-257 (batch) / construction.rs:596-601 (ring) ----
    int max_delay = 0;
    for (int p = 0; p < d->n_projections; p++)
        for (int64_t k = 0; k < d->projections[p].n_delays; k++) max_delay = std::max<int>(max_delay, (int)d->projections[p].delays[k]);
    if (max_delay > 65535) return bail(fail(HB_ERR_UNSUPPORTED, "delays above 65535 steps are not supported"));
    e->H = ring ? max_delay + 1 : (max_delay == 0 ? 0 : max_delay + 1);
    e->R = std::max(e->H, 1) + 1;  // widened below when the barrier interval allows

    // ---- projections (engine.rs:272-417) ----
    int n_mean = 0;
    for (int p = 0; p < d->n_projections; p++) {
        const hb_projection_desc& pd = d->projections[p];
        if (pd.src < 0 || pd.src >= d->n_subnets) return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: src %d >= number of subnetworks %d", p, pd.src, d->n_subnets));
        if (pd.tgt < 0 || pd.tgt >= d->n_subnets) return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: tgt %d >= number of subnetworks %d", p, pd.tgt, d->n_subnets));
        HostProj hp;
        hp.src = pd.src; hp.tgt = pd.tgt;
        const HostSub& S = e->subs[pd.src];
        const HostSub& Tg = e->subs[pd.tgt];
        hp.nsrc = S.nm; hp.ntgt = Tg.nm;
        hp.cf_name = pd.coupling_fn ? pd.coupling_fn : "Linear";
        hp.cf_params.assign(pd.coupling_params, pd.coupling_params + std::max(0, pd.n_coupling_params));
        if (hp.cf_params.size() > 16) return bail(fail(HB_ERR_UNSUPPORTED, "projection %d: too many coupling params", p));
        hp.delay = pd.n_delays > 0 ? (int)pd.delays[0] : 0;
        Cfn cf0 = resolve_cfn(hp, hp.cf_params.data(), (int)hp.cf_params.size());
        if (cf0.kind == HBC_PRESIG && cf0.global_t)
            return bail(fail(HB_ERR_UNSUPPORTED, "projection %d: PreSigmoidal global_t couples all sweep points; not supported", p));
        // weights
        std::vector<float> dense;  // only for Difference preprocessing of dense weights
        bool per_edge = false;
        if (pd.weights_kind == HB_WEIGHTS_SCALAR) {
            hp.kind = (d->flags & HB_SEM_SCALAR_DIAGONAL) ? W_DIAG : W_MEAN;
            hp.w = pd.scalar_weight;
            if (hp.kind == W_DIAG && hp.nsrc != hp.ntgt)
                return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: scalar weights require src and tgt nnodes to match (%d != %d)",
                                 p, S.nnodes, Tg.nnodes));
        } else if (pd.weights_kind == HB_WEIGHTS_DENSE) {
            if (!pd.dense) return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: dense weights pointer is NULL", p));
            if (pd.dense_rows != hp.ntgt)  // config.rs:375-380
                return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: weights has %d rows, expected %d (tgt nnodes)", p,
                                 pd.dense_rows, hp.ntgt));
            if (pd.dense_cols != hp.nsrc)  // config.rs:381-388 (every row has dense_cols entries here)
                return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: weights row 0 has %d cols, expected %d (src nnodes)", p,
                                 pd.dense_cols, hp.nsrc));
            hp.kind = W_SPARSE;
            dense.assign(pd.dense, pd.dense + (size_t)hp.ntgt * hp.nsrc);
        } else if (pd.weights_kind == HB_WEIGHTS_CSR) {
            if (pd.n_indptr != hp.ntgt + 1)
                return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: CSR indptr length %lld != tgt_nnodes + 1 = %d", p, (long long)pd.n_indptr, hp.ntgt + 1));
            if (pd.csr_indptr[0] != 0 || (int64_t)pd.csr_indptr[hp.ntgt] != pd.nnz)
                return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: CSR indptr must start at 0 and end at nnz", p));
            for (int t = 0; t < hp.ntgt; t++)
                if (pd.csr_indptr[t + 1] < pd.csr_indptr[t]) return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: CSR indptr is not monotonic", p));
            for (int64_t k = 0; k < pd.nnz; k++)
                if ((int)pd.csr_indices[k] >= hp.nsrc) return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: CSR index %u >= src nodes %d", p, pd.csr_indices[k], hp.nsrc));
            hp.kind = W_SPARSE;
            per_edge = ring && pd.n_delays == pd.nnz && pd.nnz > 0;
            if (!ring) {
                // densified by the batch engine (engine.rs:298-322)
                dense.assign((size_t)hp.ntgt * hp.nsrc, 0.0f);
                for (int t = 0; t < hp.ntgt; t++)
                    for (uint32_t k = pd.csr_indptr[t]; k < pd.csr_indptr[t + 1]; k++) dense[(size_t)t * hp.nsrc + pd.csr_indices[k]] = pd.csr_data[k];
            }
        } else return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d: unknown weights kind %d", p, pd.weights_kind));

        // Difference preprocessing (engine.rs:327-368; CSR in ring mode follows construction.rs:700-730)
        if (cf0.kind == HBC_DIFFERENCE) {
            if (hp.kind == W_MEAN || hp.kind == W_DIAG) { hp.w = 0.0f; hp.diff_mode = 1; }
            else if (!dense.empty()) {
                if (hp.ntgt == hp.nsrc) {
                    for (int i = 0; i < hp.ntgt; i++) {
                        float rs = 0.0f;
                        for (int j = 0; j < hp.nsrc; j++) rs = rs + dense[(size_t)i * hp.nsrc + j];
                        dense[(size_t)i * hp.nsrc + i] -= rs;
                    }
                    hp.diff_mode = 1;
                } else {
                    hp.rowsums.resize(hp.ntgt);
                    for (int i = 0; i < hp.ntgt; i++) {
                        float rs = 0.0f;
                        for (int j = 0; j < hp.nsrc; j++) rs = rs + dense[(size_t)i * hp.nsrc + j];
                        hp.rowsums[i] = rs;
                    }
                    hp.diff_mode = 2;
                }
            } else hp.diff_mode = 1;
        }
        hp.cf = resolve_cfn(hp, hp.cf_params.data(), (int)hp.cf_params.size());
        // CSR rows: dense rows keep only non-zero weights (exact for finite values), in source order
        if (hp.kind == W_SPARSE) {
            hp.rowptr.assign(hp.ntgt + 1, 0);
            if (!dense.empty()) {
                for (int t = 0; t < hp.ntgt; t++) {
                    for (int j = 0; j < hp.nsrc; j++) {
                        float w = dense[(size_t)t * hp.nsrc + j];
                        if (w != 0.0f) { hp.edges.push_back((uint32_t)j); hp.ew.push_back(w); }
                    }
                    hp.rowptr[t + 1] = (int)hp.edges.size();
                }
            } else {
                for (int t = 0; t < hp.ntgt; t++) {
                    for (uint32_t k = pd.csr_indptr[t]; k < pd.csr_indptr[t + 1]; k++) {
                        uint32_t dl = per_edge ? pd.delays[k] : 0;
                        hp.edges.push_back((dl << 16) | pd.csr_indices[k]);
                        hp.ew.push_back(pd.csr_data[k]);
                    }
                    hp.rowptr[t + 1] = (int)hp.edges.size();
                }
            }
        }
        hp.dmode = per_edge ? HBD_EDGE : (ring ? HBD_RING : HBD_COMPAT);
        hp.pre_cpu = per_edge ? 1 : 0;
        // channels and cvar map (engine.rs:370-392, 637-664)
        hp.ncv = std::min(S.ncvar, S.nvar);
        const Cfn& f = hp.cf;
        hp.pc = (f.kind == HBC_KURAMOTO) ? 2 * hp.ncv : ((f.kind == HBC_SJR || (f.kind == HBC_PRESIG && f.dynamic)) ? 1 : hp.ncv);
        hp.oc = (f.kind == HBC_KURAMOTO) ? Tg.ncvar : hp.pc;
        if (f.kind == HBC_PRESIG && f.dynamic && hp.ncv < 2)
            return bail(fail(HB_ERR_UNSUPPORTED, "projection %d: PreSigmoidal dynamic needs two source coupling variables", p));
        if (f.kind == HBC_KURAMOTO && hp.ncv != Tg.ncvar)
            return bail(fail(HB_ERR_UNSUPPORTED, "projection %d: Kuramoto coupling needs equal source and target cvar counts", p));
        if (hp.diff_mode == 2 && hp.pc != Tg.ncvar)
            return bail(fail(HB_ERR_UNSUPPORTED, "projection %d: Difference rowsums need equal source and target cvar counts", p));
        int cs[8], ct[8];
        int ncm = parse_cvar_map(pd.cvar_map, cs, ct, 8);
        if (ncm > 4) return bail(fail(HB_ERR_UNSUPPORTED, "projection %d: at most 4 cvar_map pairs", p));
        for (int k = 0; k < ncm; k++) {
            if (cs[k] >= S.ncvar) return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d cvar_map src index %d >= src_ncvar %d", p, cs[k], S.ncvar));
            if (ct[k] >= Tg.ncvar) return bail(fail(HB_ERR_INVALID_CONFIG, "Projection %d cvar_map tgt index %d >= tgt_ncvar %d", p, ct[k], Tg.ncvar));
            hp.cm_s[k] = cs[k];
            int pos = 0;
            if (Tg.model == HBM_MPR) pos = (ct[k] == 1) ? 1 : 0;
            else pos = (k_models[Tg.model].cvar0 == ct[k]) ? 0 : 0;
            hp.cm_cpl[k] = pos;
        }
        hp.ncm = ncm;
        hp.direct = (Tg.ncvar == S.ncvar && ncm == 1 && cs[0] == 0 && ct[0] == 0) ? 1 : 0;
        if (hp.direct && hp.oc != Tg.ncvar)
            return bail(fail(HB_ERR_UNSUPPORTED, "projection %d: coupling produces %d channels for a target with %d cvars", p, hp.oc, Tg.ncvar));
        if (!hp.direct && hp.oc != S.ncvar)
            return bail(fail(HB_ERR_UNSUPPORTED, "projection %d: cvar remap of a %d-channel coupling output", p, hp.oc));
        // device form
        DevProj& dp = e->net.proj[p];
        dp.src = hp.src; dp.tgt = hp.tgt; dp.kind = hp.kind; dp.dmode = hp.dmode; dp.delay = hp.delay;
        dp.nsrc = hp.nsrc; dp.ntgt = hp.ntgt; dp.cfk = f.kind; dp.pre_cpu = hp.pre_cpu; dp.ncv = hp.ncv; dp.pc = hp.pc;
        dp.oc = hp.oc; dp.has_rowsums = hp.diff_mode == 2; dp.direct = hp.direct; dp.ncm = ncm;
        for (int k = 0; k < 4; k++) { dp.cm_s[k] = hp.cm_s[k]; dp.cm_cpl[k] = hp.cm_cpl[k]; }
        dp.w = hp.w;
        cfn_to_cp(f, hp.nsrc, dp.cp);
        dp.mean_slot = (hp.kind == W_MEAN) ? n_mean++ : -1;
        e->projs.push_back(hp);
    }
    e->n_mean = n_mean;
    for (int i = 0; i < d->n_subnets; i++) {
        DevSub& ds = e->net.sub[i];
        ds.n_in = 0;
        ds.n_mean_out = 0;
        for (int p = 0; p < d->n_projections; p++) {
            if (e->projs[p].tgt == i) {
                if (ds.n_in == HB_MAX_IN)
                    return bail(fail(HB_ERR_UNSUPPORTED, "subnetwork %d receives more than %d projections", i, HB_MAX_IN));
                ds.in_idx[ds.n_in++] = p;
            }
            if (e->projs[p].src == i && e->projs[p].kind == W_MEAN) ds.mean_out[ds.n_mean_out++] = p;
        }
        ds.integ = eff_integrator(e, e->subs[i].model);
    }
    // Barrier interval of the specialised kernel: one subnetwork, one sparse projection with
    // per-edge delays, all >= 1. The ring then needs H + K slots; K shrinks (to 1) when the wider
    // ring would no longer fit the shared-memory budget that fits it at K = 1.
    if (d->n_subnets == 1 && d->n_projections == 1 && e->projs[0].kind == W_SPARSE &&
        (e->projs[0].dmode == HBD_EDGE || (e->projs[0].dmode == HBD_RING && e->projs[0].delay > 0))) {
        int dmin = 1 << 30;
        if (e->projs[0].dmode == HBD_EDGE) {
            for (uint32_t m : e->projs[0].edges) dmin = std::min(dmin, (int)(m >> 16));
            if (e->projs[0].edges.empty()) dmin = 1;
        } else dmin = e->projs[0].delay;
        e->dmin = dmin;
        int K = std::max(1, std::min(dmin, 32));
        const size_t budget = 216 * 1024, edges_b = e->projs[0].edges.size() * 8;
        auto fits = [&](int k) { return (size_t)(std::max(e->H, 1) + k) * e->cols * 4 + edges_b <= budget; };
        if (fits(1)) while (K > 1 && !fits(K)) K >>= 1;
        e->sync_every = K;
        // the warp-specialised pipeline needs H + 2 * 8 slots
        const int want = std::max(K, dmin >= 15 ? 16 : 1);
        e->R = std::max(e->H, 1) + want;
    }
    e->net.R = e->R;
    e->kernel_model = e->subs[0].model;
    for (auto& sb : e->subs)
        if (sb.model != e->kernel_model) e->kernel_model = -1;
    // ring offset of every edge: source column minus delay * cols (per-edge) or the source column
    for (auto& hp : e->projs) {
        if (hp.kind != W_SPARSE) continue;
        const int scol = e->net.sub[hp.src].col_off, sncv = e->subs[hp.src].ncvar;
        hp.eoff.resize(hp.edges.size());
        for (size_t k2 = 0; k2 < hp.edges.size(); k2++) {
            int src = (int)(hp.edges[k2] & 0xffffu), dl = (int)(hp.edges[k2] >> 16);
            hp.eoff[k2] = scol + src * sncv - (hp.dmode == HBD_EDGE ? dl * e->cols : 0);
            hp.maxd = std::max(hp.maxd, dl);
        }
    }
    for (size_t p = 0; p < e->projs.size(); p++) e->net.proj[p].maxd = e->projs[p].maxd;
    // BOLD monitors (engine.rs:419-449)
    for (int m = 0; m < d->n_bold; m++) {
        if (e->subs[0].nmodes != 1) return bail(fail(HB_ERR_UNSUPPORTED, "BOLD monitors need nmodes == 1 on subnetwork 0"));
        e->bold_cfg.push_back(d->bold[m]);
        BoldHost bh;
        bh.period = std::max(1, d->bold[m].bold_period);
        bh.tr = d->bold[m].tr;
        e->bold.push_back(std::move(bh));
    }
    // network-wide constants
    DevNet& net = e->net;
    net.n_sub = d->n_subnets; net.n_proj = d->n_projections; net.n_mean = n_mean;
    net.B = e->B; net.H = e->H; net.R = e->R; net.cols = e->cols; net.state_len = e->state_len; net.noise_row = e->noise_row;
    const float dt = (float)d->dt;
    net.dt = dt; net.dt_half = dt * 0.5f; net.dt_sixth = dt / 6.0f; net.dt_h2 = dt / 2.0f;
    const float sqrt_dt = sqrtf(dt);
    for (int v = 0; v < 8; v++) net.noise_scale[v] = v < (int)e->nsig.size() ? sqrtf(2.0f * e->nsig[v]) * sqrt_dt : 0.0f;

    // ---- device allocations ----
    auto cu = [&](cudaError_t err, const char* what) -> hb_status {
        if (err != cudaSuccess) return fail(HB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
        return HB_OK;
    };
    hb_status s;
    if ((s = cu(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking), "cudaStreamCreate"))) return bail(s);
    if ((s = cu(cudaEventCreate(&e->ev0), "cudaEventCreate"))) return bail(s);
    if ((s = cu(cudaEventCreate(&e->ev1), "cudaEventCreate"))) return bail(s);
    if ((s = cu(cudaMalloc(&e->d_net, sizeof(DevNet)), "cudaMalloc(net)"))) return bail(s);
    const size_t stn = (size_t)e->B * e->state_len;
    if ((s = cu(e->state.ensure(stn), "cudaMalloc(state)"))) return bail(s);
    if ((s = cu(e->x0.ensure(stn), "cudaMalloc(x0)"))) return bail(s);
    if ((s = cu(e->tavg.ensure(stn), "cudaMalloc(tavg)"))) return bail(s);
    if ((s = cu(e->ring.ensure((size_t)e->B * (((size_t)e->R * e->cols + 3) & ~(size_t)3)), "cudaMalloc(ring)"))) return bail(s);
    {
        std::vector<float> x0(stn);
        for (int b = 0; b < e->B; b++)
            for (size_t i = 0; i < e->subs.size(); i++)
                memcpy(&x0[(size_t)b * e->state_len + e->net.sub[i].state_off], e->subs[i].x0.data(), e->subs[i].x0.size() * 4);
        if ((s = cu(cudaMemcpy(e->x0.p, x0.data(), stn * 4, cudaMemcpyHostToDevice), "upload x0"))) return bail(s);
        if ((s = cu(cudaMemcpy(e->state.p, x0.data(), stn * 4, cudaMemcpyHostToDevice), "upload state"))) return bail(s);
    }
    e->d_params.resize(e->subs.size());
    e->d_node_params.resize(e->subs.size());
    for (size_t p = 0; p < e->projs.size(); p++) {
        HostProj& hp = e->projs[p];
        DevProj& dp = e->net.proj[p];
        if (hp.kind == W_SPARSE) {
            if ((s = cu(cudaMalloc(&hp.d_rowptr, hp.rowptr.size() * 4), "cudaMalloc(rowptr)"))) return bail(s);
            if ((s = cu(cudaMemcpy(hp.d_rowptr, hp.rowptr.data(), hp.rowptr.size() * 4, cudaMemcpyHostToDevice), "upload rowptr"))) return bail(s);
            size_t ne = std::max<size_t>(hp.edges.size(), 1);
            if ((s = cu(cudaMalloc(&hp.d_edges, ne * 4), "cudaMalloc(edges)"))) return bail(s);
            if ((s = cu(cudaMalloc(&hp.d_eoff, ne * 4), "cudaMalloc(eoff)"))) return bail(s);
            if ((s = cu(cudaMalloc(&hp.d_ew, ne * 4), "cudaMalloc(ew)"))) return bail(s);
            if (!hp.edges.empty()) {
                if ((s = cu(cudaMemcpy(hp.d_edges, hp.edges.data(), hp.edges.size() * 4, cudaMemcpyHostToDevice), "upload edges"))) return bail(s);
                if ((s = cu(cudaMemcpy(hp.d_eoff, hp.eoff.data(), hp.eoff.size() * 4, cudaMemcpyHostToDevice), "upload eoff"))) return bail(s);
                if ((s = cu(cudaMemcpy(hp.d_ew, hp.ew.data(), hp.ew.size() * 4, cudaMemcpyHostToDevice), "upload weights"))) return bail(s);
            }
            dp.rowptr = hp.d_rowptr; dp.edges = hp.d_edges; dp.eoff = hp.d_eoff; dp.ew = hp.d_ew;
        }
        if (!hp.rowsums.empty()) {
            if ((s = cu(cudaMalloc(&hp.d_rowsums, hp.rowsums.size() * 4), "cudaMalloc(rowsums)"))) return bail(s);
            if ((s = cu(cudaMemcpy(hp.d_rowsums, hp.rowsums.data(), hp.rowsums.size() * 4, cudaMemcpyHostToDevice), "upload rowsums"))) return bail(s);
            dp.rowsums = hp.d_rowsums;
        }
    }
    if ((s = reset_bold_device(e))) return bail(s);
    *out = e;
    return HB_OK;
}

void hb_engine_destroy(hb_engine* e) {
    if (!e) return;
    if (e->own_stream) cudaStreamSynchronize(e->own_stream);
    for (auto& hp : e->projs) {
        if (hp.d_rowptr) cudaFree(hp.d_rowptr);
        if (hp.d_edges) cudaFree(hp.d_edges);
        if (hp.d_eoff) cudaFree(hp.d_eoff);
        if (hp.d_ew) cudaFree(hp.d_ew);
        if (hp.d_rowsums) cudaFree(hp.d_rowsums);
        if (hp.d_cp_pp) cudaFree(hp.d_cp_pp);
    }
    for (auto& b : e->d_params) b.release();
    for (auto& b : e->d_node_params) b.release();
    for (auto& bh : e->bold) { bh.bw.release(); bh.acc.release(); bh.win.release(); bh.out_run.release(); bh.emit.release(); }
    e->state.release(); e->x0.release(); e->tavg.release(); e->ring.release(); e->noise.release(); e->prep_noise.release();
    e->traj.release(); e->dtraj.release();
    e->fe_fc.release(); e->fe_feat.release(); e->fe_fcd.release(); e->fe_fcds.release(); e->fe_ut.release();
    e->fe_part.release(); e->fe_mv.release();
    e->means.release(); e->flags_buf.release(); e->porder.release(); e->dtc.release();
    if (e->d_net) cudaFree(e->d_net);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    if (e->own_stream) cudaStreamDestroy(e->own_stream);
    delete e;
}

static hb_status run_common(hb_engine* e, const hb_sweep_point* dims, int n_dims, bool multi, int64_t n_steps,
                            uint32_t run_flags, const float* noise, int64_t noise_len, hb_result** out) {
    if (!e || !out) return fail(HB_ERR_INVALID_STATE, "NULL engine or result pointer");
    *out = nullptr;
    if (n_steps < 1) return fail(HB_ERR_INVALID_STATE, "n_steps must be >= 1");
    hb_status s = validate_noise(e, noise, noise_len, n_steps);
    if (s) return s;
    RunTables T;
    if ((s = build_tables(e, dims, n_dims, multi, T))) return s;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    cudaEventRecord(t0, e->stream());
    hb_result* r = new hb_result();
    if (multi) {
        // a fresh engine seeded by sweep point 0's current state, without BOLD (engine.rs:886-915)
        cudaStream_t st = e->stream();
        for (int b = 1; b < e->B; b++) {
            cudaError_t err = cudaMemcpyAsync(e->state.p + (size_t)b * e->state_len, e->state.p, e->state_len * 4, cudaMemcpyDeviceToDevice, st);
            if (err != cudaSuccess) { delete r; return fail(HB_ERR_CUDA, "reseed: %s", cudaGetErrorString(err)); }
        }
        e->step = 0;
        e->bold_removed = true;
    }
    s = run_device(e, T, n_steps, run_flags, noise, nullptr, r);
    if (!s) s = collect(e, n_steps, r);
    cudaEventRecord(t1, e->stream());
    cudaEventSynchronize(t1);
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (s) { delete r; return s; }
    r->elapsed_ms = ms;
    r->params = T.param_values;
    r->has_traj = (run_flags & HB_RUN_TRAJECTORY) != 0;
    *out = r;
    return HB_OK;
}

hb_status hb_engine_run_sweep(hb_engine* e, int32_t sub_idx, int32_t param_idx, const float* values, int32_t n_values,
                              int64_t n_steps, uint32_t run_flags, const float* noise, int64_t noise_len, hb_result** out) {
    if (!e) return fail(HB_ERR_INVALID_STATE, "NULL engine");
    if (n_values != e->B || !values) return fail(HB_ERR_INVALID_STATE, "expected %d sweep values, got %d", e->B, n_values);
    hb_sweep_point dim{sub_idx, param_idx, values, n_values};
    return run_common(e, &dim, 1, false, n_steps, run_flags, noise, noise_len, out);
}

hb_status hb_engine_run_sweep_multi(hb_engine* e, const hb_sweep_point* dims, int32_t n_dims, int64_t n_steps,
                                    uint32_t run_flags, const float* noise, int64_t noise_len, hb_result** out) {
    if (!e) return fail(HB_ERR_INVALID_STATE, "NULL engine");
    if (!dims || n_dims < 1) return fail(HB_ERR_INVALID_STATE, "empty sweep");
    int64_t n = 1;
    for (int d = 0; d < n_dims; d++) n *= dims[d].n_values;
    if (n != e->B) return fail(HB_ERR_INVALID_STATE, "Cartesian product has %lld points, engine has %d", (long long)n, e->B);
    return run_common(e, dims, n_dims, true, n_steps, run_flags, noise, noise_len, out);
}

hb_status hb_engine_get_state(hb_engine* e, int32_t sub_idx, float* out, int64_t len) {
    if (!e || !out) return fail(HB_ERR_INVALID_STATE, "NULL argument");
    if (sub_idx < 0 || sub_idx >= (int)e->subs.size()) return fail(HB_ERR_INVALID_CONFIG, "subnetwork index %d out of range", sub_idx);
    const int per = e->subs[sub_idx].nm * e->subs[sub_idx].nvar;
    if (len < (int64_t)e->B * per) return fail(HB_ERR_INVALID_STATE, "output buffer too small");
    std::vector<float> st((size_t)e->B * e->state_len);
    CUDA_TRY(cudaMemcpyAsync(st.data(), e->state.p, st.size() * 4, cudaMemcpyDeviceToHost, e->stream()));
    CUDA_TRY(cudaStreamSynchronize(e->stream()));
    for (int b = 0; b < e->B; b++) memcpy(out + (size_t)b * per, &st[(size_t)b * e->state_len + e->net.sub[sub_idx].state_off], per * 4);
    return HB_OK;
}

int64_t hb_engine_step(const hb_engine* e) { return e ? e->step : -1; }

hb_status hb_engine_reset(hb_engine* e) {
    if (!e) return fail(HB_ERR_INVALID_STATE, "NULL engine");
    hb_status s = reset_state(e);
    if (s) return s;
    e->bold_removed = false;
    return reset_bold_device(e);
}

hb_status hb_engine_last_kernel_time(const hb_engine* e, double* ms, int64_t* launches, int32_t* kind) {
    if (!e) return fail(HB_ERR_INVALID_STATE, "NULL engine");
    if (ms) *ms = e->last_ms;
    if (launches) *launches = e->last_launches;
    if (kind) *kind = e->last_kind;
    return HB_OK;
}

hb_status hb_engine_set_hybrid_integrator(hb_engine* e, int32_t on) {
    if (!e) return fail(HB_ERR_INVALID_STATE, "NULL engine");
    if (on) e->flags |= HB_SEM_HYBRID_INTEGRATOR;
    else e->flags &= ~(uint32_t)HB_SEM_HYBRID_INTEGRATOR;
    // each subnetwork's integrator in the device network (uploaded with the tables of every run)
    for (size_t i = 0; i < e->subs.size(); i++) e->net.sub[i].integ = eff_integrator(e, e->subs[i].model);
    return HB_OK;
}

hb_status hb_engine_set_stream(hb_engine* e, void* stream) {
    if (!e) return fail(HB_ERR_INVALID_STATE, "NULL engine");
    if (e->own_stream) CUDA_TRY(cudaStreamSynchronize(e->own_stream));
    e->user_stream = (cudaStream_t)stream;
    return HB_OK;
}

hb_status hb_engine_prepare(hb_engine* e, int32_t sub_idx, int32_t param_idx, const float* values, int32_t n_values,
                            int64_t n_steps, uint32_t run_flags, const float* noise, int64_t noise_len) {
    if (!e) return fail(HB_ERR_INVALID_STATE, "NULL engine");
    if (n_values != e->B || !values) return fail(HB_ERR_INVALID_STATE, "expected %d sweep values, got %d", e->B, n_values);
    if (n_steps < 1) return fail(HB_ERR_INVALID_STATE, "n_steps must be >= 1");
    hb_status s = validate_noise(e, noise, noise_len, n_steps);
    if (s) return s;
    hb_sweep_point dim{sub_idx, param_idx, values, n_values};
    if ((s = build_tables(e, &dim, 1, false, e->prep_tables))) return s;
    e->prep_steps = n_steps;
    e->prep_flags = run_flags & ~HB_RUN_TRAJECTORY;
    e->prep_noise_len = noise ? noise_len : 0;
    if (noise) {
        CUDA_TRY(e->prep_noise.ensure((size_t)noise_len));
        CUDA_TRY(cudaMemcpy(e->prep_noise.p, noise, (size_t)noise_len * 4, cudaMemcpyHostToDevice));
    }
    e->prepared = true;
    return HB_OK;
}

hb_status hb_engine_execute_prepared(hb_engine* e) {
    if (!e || !e->prepared) return fail(HB_ERR_INVALID_STATE, "no prepared run");
    hb_status s = reset_state(e);
    if (s) return s;
    e->bold_removed = false;
    if ((s = reset_bold_device(e))) return s;
    return run_device(e, e->prep_tables, e->prep_steps, e->prep_flags, nullptr,
                      e->prep_noise_len ? e->prep_noise.p : e->x0.p, nullptr);
}

int32_t hb_result_n_sweep(const hb_result* r) { return r ? r->n_sweep : 0; }
int32_t hb_result_n_subnets(const hb_result* r) { return r ? (int32_t)r->tavg.size() : 0; }
int32_t hb_result_n_bold(const hb_result* r) { return r ? r->n_bold : 0; }
double hb_result_elapsed_ms(const hb_result* r) { return r ? r->elapsed_ms : 0.0; }
const float* hb_result_param_values(const hb_result* r, int64_t* len) {
    if (len) *len = r ? (int64_t)r->params.size() : 0;
    return r && !r->params.empty() ? r->params.data() : nullptr;
}
#define RESULT_VEC(fn, member)                                                             \
    const float* fn(const hb_result* r, int32_t i, int64_t* len) {                         \
        if (len) *len = 0;                                                                 \
        if (!r || i < 0 || i >= (int32_t)r->member.size()) return nullptr;                  \
        if (len) *len = (int64_t)r->member[i].size();                                      \
        return r->member[i].data();                                                        \
    }
RESULT_VEC(hb_result_tavg, tavg)
RESULT_VEC(hb_result_final_states, fin)
RESULT_VEC(hb_result_bold, bold)
const float* hb_result_trajectory(const hb_result* r, int32_t i, int64_t* len) {
    if (len) *len = 0;
    if (!r || !r->has_traj || i < 0 || i >= (int32_t)r->traj.size()) return nullptr;
    if (len) *len = (int64_t)r->traj[i].size();
    return r->traj[i].data();
}
hb_status hb_engine_adjoint_order(hb_engine* e, const float* gain_values, int32_t n_values, int64_t n_steps,
                                  uint32_t run_flags, hb_order_adjoint_out* out) {
    if (!e || !gain_values || !out) return fail(HB_ERR_INVALID_STATE, "NULL argument");
    if (n_values != e->B) return fail(HB_ERR_INVALID_STATE, "expected %d gain values, got %d", e->B, n_values);
    if (n_steps < 2 || n_steps > (1 << 28)) return fail(HB_ERR_INVALID_STATE, "n_steps must be in [2, 2^28]");
    if (e->subs.size() != 1 || e->projs.size() != 1 || e->subs[0].model != HBM_KURAMOTO || e->subs[0].nmodes != 1)
        return fail(HB_ERR_UNSUPPORTED, "the order-parameter adjoint needs one Kuramoto subnetwork (one mode) and one projection");
    HostProj& hp = e->projs[0];
    if (hp.kind != W_SPARSE || hp.dmode != HBD_EDGE || hp.cf.kind != HBC_KURAMOTO || hp.ncv != 1)
        return fail(HB_ERR_UNSUPPORTED, "the order-parameter adjoint needs Kuramoto coupling through a CSR projection with "
                    "per-edge delays (HB_SEM_DELAY_RING)");
    if (eff_integrator(e, HBM_KURAMOTO) != HBI_HEUN_DET)
        return fail(HB_ERR_UNSUPPORTED, "the order-parameter adjoint differentiates deterministic Heun");
    const int N = e->subs[0].nm, B = e->B, T = (int)n_steps;
    if (N > 1024) return fail(HB_ERR_UNSUPPORTED, "the order-parameter adjoint supports up to 1024 nodes");
    int dmin = 1 << 30;
    for (uint32_t m : hp.edges) dmin = std::min(dmin, (int)(m >> 16));
    if (hp.edges.empty()) dmin = 8;
    if (dmin < 1) return fail(HB_ERR_UNSUPPORTED, "the order-parameter adjoint needs every edge delay >= 1");
    const int K = std::min(dmin, 8);
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const double need = (double)B * N * ((double)(T + 1) * 8 + (double)T * 8 + (double)T * 4 + (double)T * 8) +
                        (double)B * T * 8;
    if (need > 0.8 * (double)free_b)
        return fail(HB_ERR_UNSUPPORTED, "the order-parameter adjoint needs %.2f GB of device memory, %.2f GB free", need / 1e9,
                    free_b / 1e9);
    // forward: the engine's own run from its initial state, every step's phase kept on the device
    // (the pipeline and streamed-history kernels also write the coupling sums S, C of every step)
    DBuf<float> d_cs;
    CUDA_TRY(d_cs.ensure((size_t)T * B * N * 2));
    hb_status s = hb_engine_reset(e);
    if (s) return s;
    hb_result* res = nullptr;
    e->cs_out = d_cs.p;
    s = hb_engine_run_sweep(e, -1, 0, gain_values, n_values, n_steps,
                            (run_flags & ~HB_RUN_TRAJECTORY) | HB_RUN_DEVICE_TRAJECTORY, nullptr, 0, &res);
    e->cs_out = nullptr;
    if (s) return s;
    hb_result_free(res);
    const float forward_ms = (float)e->last_ms;
    const bool have_cs = e->last_kind == 3 || e->last_kind == 4;
    // out-edges of every source node (transpose of the CSR rows)
    std::vector<int> cptr(N + 1, 0), ctgt(hp.edges.size()), cdel(hp.edges.size());
    std::vector<float> cw(hp.edges.size()), kh(B);
    for (uint32_t m : hp.edges) cptr[(m & 0xffffu) + 1]++;
    for (int j = 0; j < N; j++) cptr[j + 1] += cptr[j];
    {
        std::vector<int> fill(cptr.begin(), cptr.end() - 1);
        for (int i = 0; i < N; i++)
            for (int q = hp.rowptr[i]; q < hp.rowptr[i + 1]; q++) {
                const int src = (int)(hp.edges[q] & 0xffffu), c = fill[src]++;
                ctgt[c] = i; cdel[c] = (int)(hp.edges[q] >> 16); cw[c] = hp.ew[q];
            }
    }
    // the coupling's a / N as the engine resolves it for each point
    for (int b = 0; b < B; b++) kh[b] = gain_values[b] / (float)hp.nsrc;
    DBuf<int> d_cptr, d_ctgt, d_cdel;
    DBuf<float> d_cw, d_k, d_sc, d_z, d_nu;
    DBuf<double> d_loss, d_gA, d_gW, d_gWn;
    cudaStream_t st = e->stream();
    const size_t nnz = std::max<size_t>(hp.edges.size(), 1);
    CUDA_TRY(d_cptr.ensure(N + 1)); CUDA_TRY(d_ctgt.ensure(nnz)); CUDA_TRY(d_cdel.ensure(nnz)); CUDA_TRY(d_cw.ensure(nnz));
    CUDA_TRY(d_k.ensure(B));
    CUDA_TRY(d_sc.ensure((size_t)B * N * (T + 1) * 2)); CUDA_TRY(d_z.ensure((size_t)B * T * 2));
    CUDA_TRY(d_nu.ensure((size_t)B * N * T * 2));
    CUDA_TRY(d_loss.ensure(B)); CUDA_TRY(d_gA.ensure(B)); CUDA_TRY(d_gW.ensure(B)); CUDA_TRY(d_gWn.ensure((size_t)B * N));
    CUDA_TRY(cudaMemcpyAsync(d_cptr.p, cptr.data(), (N + 1) * 4, cudaMemcpyHostToDevice, st));
    if (!hp.edges.empty()) {
        CUDA_TRY(cudaMemcpyAsync(d_ctgt.p, ctgt.data(), ctgt.size() * 4, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(d_cdel.p, cdel.data(), cdel.size() * 4, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(d_cw.p, cw.data(), cw.size() * 4, cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(cudaMemcpyAsync(d_k.p, kh.data(), B * 4, cudaMemcpyHostToDevice, st));
    HbKuraAdjLaunch L;
    memset(&L, 0, sizeof L);
    L.traj = e->dtraj.p; L.x0 = e->x0.p; L.B = B; L.N = N; L.T = T; L.K = K; L.dt = e->net.dt; L.k = d_k.p;
    L.maxd = hp.maxd;
    L.rowptr = hp.d_rowptr; L.edges = hp.d_edges; L.ew = hp.d_ew;
    L.cptr = d_cptr.p; L.ctgt = d_ctgt.p; L.cdel = d_cdel.p; L.cw = d_cw.p;
    L.sc = d_sc.p; L.z = d_z.p; L.nu = d_nu.p; L.loss = d_loss.p; L.gA = d_gA.p; L.gW = d_gW.p; L.gWn = d_gWn.p;
    L.cs = have_cs ? d_cs.p : nullptr;
    cudaEvent_t ev[3];
    for (auto& v : ev) CUDA_TRY(cudaEventCreate(&v));
    cudaError_t ce = cudaEventRecord(ev[0], st);
    if (ce == cudaSuccess) ce = hb_launch_kura_adjoint(L, 0, st);
    if (ce == cudaSuccess) ce = cudaEventRecord(ev[1], st);
    if (ce == cudaSuccess) ce = hb_launch_kura_adjoint(L, 1, st);
    if (ce == cudaSuccess) ce = cudaEventRecord(ev[2], st);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(ev[2]);
    float ms[2] = {0, 0};
    for (int q = 0; q < 2 && ce == cudaSuccess; q++) ce = cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]);
    for (auto& v : ev) cudaEventDestroy(v);
    if (ce != cudaSuccess) return fail(HB_ERR_CUDA, "order-parameter adjoint: %s", cudaGetErrorString(ce));
    if (out->loss) CUDA_TRY(cudaMemcpy(out->loss, d_loss.p, B * 8, cudaMemcpyDeviceToHost));
    if (out->d_gain) CUDA_TRY(cudaMemcpy(out->d_gain, d_gA.p, B * 8, cudaMemcpyDeviceToHost));
    if (out->d_omega) CUDA_TRY(cudaMemcpy(out->d_omega, d_gW.p, B * 8, cudaMemcpyDeviceToHost));
    if (out->d_omega_node) CUDA_TRY(cudaMemcpy(out->d_omega_node, d_gWn.p, (size_t)B * N * 8, cudaMemcpyDeviceToHost));
    out->forward_ms = forward_ms;
    out->prepare_ms = ms[0];
    out->reverse_ms = ms[1];
    return HB_OK;
}

hb_status hb_engine_fc_features(hb_engine* e, int32_t sub_idx, int32_t window_len, int32_t stride, hb_fc_features* out) {
    if (!e || !out) return fail(HB_ERR_INVALID_STATE, "hb_engine_fc_features: null argument");
    if (sub_idx < 0 || sub_idx >= (int32_t)e->subs.size()) return fail(HB_ERR_INVALID_STATE, "subnetwork index %d out of range", sub_idx);
    const int64_t T64 = e->dtraj_steps;
    if (T64 < 1) return fail(HB_ERR_INVALID_STATE, "the last run kept no device trajectory (run with HB_RUN_DEVICE_TRAJECTORY)");
    if (T64 > INT32_MAX / 2) return fail(HB_ERR_UNSUPPORTED, "device trajectory of %lld steps is too long for the features", (long long)T64);
    const int T = (int)T64;
    const HostSub& sb = e->subs[sub_idx];
    const int N = sb.nnodes, nvar = sb.nvar, B = e->B;
    if (N > 1024) return fail(HB_ERR_UNSUPPORTED, "FC features support up to 1024 nodes, got %d", N);
    int nw = 0;
    if (window_len != 0) {
        if (window_len < 2 || window_len > T) return fail(HB_ERR_INVALID_STATE, "window_len must be in [2, n_steps]");
        if (stride < 1) return fail(HB_ERR_INVALID_STATE, "stride must be > 0");
        nw = (T - window_len) / stride + 1;
        if (nw <= 1) nw = 0;
        if (nw > 32768) return fail(HB_ERR_UNSUPPORTED, "%d FCD windows; at most 32768 are supported", nw);
    }
    if (!out->fc && !out->features && !out->fcd && !out->fcd_stats) {  // size query
        out->n_windows = nw; out->nnodes = N; out->nvar = nvar; out->ms = 0.0f;
        return HB_OK;
    }
    const size_t pl = hb_fc_part_len(N), n_ut = (size_t)N * (N - 1) / 2;
    // slices of the moment passes: enough blocks to fill the SMs, each slice at least 64 steps
    const int fc_slices = std::max(1, std::min({16, (4 * 456 + B * nvar - 1) / (B * nvar), std::max(1, T / 64)}));
    const int win_slices = nw ? std::max(1, std::min({8, (456 + B * nvar * nw - 1) / (B * nvar * nw),
                                                      std::max(1, window_len / 64), 65535 / nw})) : 1;
    // FCD from blocks of G = gcd(window, stride) steps when G >= 64 and a window spans at most 12
    int block_len = 0, n_blocks = 0;
    if (nw) {
        int g = window_len, h = stride;
        while (h) { const int t = g % h; g = h; h = t; }
        if (g >= 64 && window_len / g <= 12 && N <= 512) {
            block_len = g;
            n_blocks = (nw - 1) * (stride / g) + window_len / g;
        }
    }
    const size_t win_ranges = block_len ? (size_t)n_blocks : (size_t)nw * win_slices;
    // points per batch: moments and window workspaces within 4 GiB
    const size_t per_point = (size_t)nvar * (std::max<size_t>((size_t)fc_slices, win_ranges) * pl * 8 +
                                             (size_t)nw * (n_ut * 4 + 16));
    const int nb = (int)std::max<size_t>(1, std::min<size_t>((size_t)B, (4ull << 30) / std::max<size_t>(per_point, 1)));
    CUDA_TRY(e->fe_fc.ensure((size_t)B * nvar * N * N));
    CUDA_TRY(e->fe_feat.ensure((size_t)B * nvar * 7));
    CUDA_TRY(e->fe_fcd.ensure((size_t)B * nvar * std::max(nw, 1) * std::max(nw, 1)));
    CUDA_TRY(e->fe_fcds.ensure((size_t)B * nvar * 5));
    HbFeatLaunch L;
    memset(&L, 0, sizeof L);
    L.traj = e->dtraj.p; L.T = T; L.B = B; L.state_len = e->state_len; L.off = e->net.sub[sub_idx].state_off;
    L.nnodes = N; L.nmodes = sb.nmodes; L.nvar = nvar;
    L.window = window_len; L.stride = stride; L.n_windows = nw;
    L.fc = e->fe_fc.p; L.feat = e->fe_feat.p; L.fcd = e->fe_fcd.p; L.fcd_stats = e->fe_fcds.p;
    L.fc_slices = fc_slices;
    L.win_slices = win_slices;
    L.block_len = block_len;
    const size_t part_n = (size_t)nb * nvar * std::max<size_t>((size_t)L.fc_slices, win_ranges) * pl;
    CUDA_TRY(e->fe_part.ensure(part_n));
    L.part = e->fe_part.p;
    if (nw) {
        CUDA_TRY(e->fe_ut.ensure((size_t)nb * nvar * nw * std::max<size_t>(n_ut, 1)));
        CUDA_TRY(e->fe_mv.ensure((size_t)nb * nvar * nw * 2));
        L.ut = e->fe_ut.p;
        L.ut_mv = e->fe_mv.p;
    }
    cudaStream_t st = e->stream();
    CUDA_TRY(cudaEventRecord(e->ev0, st));
    for (int b0 = 0; b0 < B; b0 += nb) {
        L.b0 = b0;
        L.nb = std::min(nb, B - b0);
        CUDA_TRY(hb_launch_fc_features(L, st));
    }
    CUDA_TRY(cudaEventRecord(e->ev1, st));
    const size_t nbv = (size_t)B * nvar;
    if (out->fc) CUDA_TRY(cudaMemcpyAsync(out->fc, e->fe_fc.p, nbv * N * N * 4, cudaMemcpyDeviceToHost, st));
    if (out->features) CUDA_TRY(cudaMemcpyAsync(out->features, e->fe_feat.p, nbv * 7 * 4, cudaMemcpyDeviceToHost, st));
    if (out->fcd && nw) CUDA_TRY(cudaMemcpyAsync(out->fcd, e->fe_fcd.p, nbv * nw * nw * 4, cudaMemcpyDeviceToHost, st));
    if (out->fcd_stats && nw) CUDA_TRY(cudaMemcpyAsync(out->fcd_stats, e->fe_fcds.p, nbv * 5 * 4, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (out->fcd_stats && !nw)
        for (size_t i = 0; i < nbv * 5; i++) out->fcd_stats[i] = std::numeric_limits<float>::quiet_NaN();
    float ms = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    out->ms = ms;
    out->n_windows = nw;
    out->nnodes = N;
    out->nvar = nvar;
    return HB_OK;
}

hb_status hb_engine_write_tavg(const hb_engine* e, const hb_result* r, const char* output_dir) {
    if (!e || !r || !output_dir) return fail(HB_ERR_INVALID_STATE, "hb_engine_write_tavg: null argument");
    if (r->tavg.size() > e->subs.size()) return fail(HB_ERR_INVALID_STATE, "result has more subnetworks than the engine");
    hb_status s = hb_io_make_dirs(output_dir);
    if (s) return s;
    for (size_t i = 0; i < r->tavg.size(); i++) {
        // the shape label [n_sweep, nvar, nnodes*nmodes] of cli.rs:961-970 over data laid out
        // [n_sweep, nnodes*nmodes, nvar]
        const std::vector<int64_t> shape = {r->n_sweep, e->subs[i].nvar, e->subs[i].nm};
        if ((int64_t)r->tavg[i].size() != shape[0] * shape[1] * shape[2])
            return fail(HB_ERR_INVALID_STATE, "tavg of subnetwork %zu does not match the engine's shape", i);
        s = hb_io_write_npy(std::string(output_dir) + "/tavg_sub" + std::to_string(i) + ".npy", r->tavg[i].data(), shape);
        if (s) return s;
    }
    return HB_OK;
}

void hb_result_free(hb_result* r) { delete r; }

}  // extern "C"

// ======================================================================================
// Grouped launch: several engines' sweeps in one kernel launch, replayed from a CUDA graph
// ======================================================================================

struct hb_group {
    struct Member {
        hb_engine* e = nullptr;
        RunTables T;
        RunPlan P;
        DBuf<float> noise;
        std::vector<DBuf<float>> bw_init;  // per BOLD monitor: the Balloon-Windkessel start state
    };
    std::vector<Member> m;
    DBuf<StreamJob> jobs;
    DBuf<int> counter;   // the work queue's next item
    cudaStream_t own = nullptr, user = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0;
    bool executed = false;
    cudaStream_t stream() const { return user ? user : own; }
    ~hb_group() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        for (auto& mm : m) { mm.noise.release(); for (auto& b : mm.bw_init) b.release(); }
        jobs.release();
        counter.release();
        if (own) cudaStreamDestroy(own);
    }
};

hb_status hb_group_prepare(const hb_group_member* members, int32_t n, void* cuda_stream, hb_group** out) {
    if (!members || n < 1 || !out) return fail(HB_ERR_INVALID_STATE, "empty group");
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        if (!members[i].engine) return fail(HB_ERR_INVALID_STATE, "group member %d has no engine", i);
        for (int j = 0; j < i; j++)
            if (members[j].engine == members[i].engine) return fail(HB_ERR_INVALID_STATE, "engine of member %d appears twice", i);
        if (members[i].run_flags & HB_RUN_TRAJECTORY) return fail(HB_ERR_UNSUPPORTED, "grouped launches record no trajectories");
        if (members[i].n_steps < 1) return fail(HB_ERR_INVALID_STATE, "member %d: n_steps must be >= 1", i);
        if (members[i].n_values != members[i].engine->B || !members[i].values)
            return fail(HB_ERR_INVALID_STATE, "member %d: expected %d sweep values", i, members[i].engine->B);
    }
    // one kernel instantiation for all: nodes per consumer thread from the largest member
    int max_nm = 0;
    for (int i = 0; i < n; i++) max_nm = std::max(max_nm, members[i].engine->subs[0].nm);
    // four nodes per consumer thread (768 threads) when every member asks for it
    bool want4 = true;
    for (int i = 0; i < n; i++) want4 = want4 && ((members[i].run_flags >> 24) & 0x7) == 4;
    const int npt = want4 && max_nm <= 2048 ? 4 : max_nm <= 96 ? 1 : 2;
    const int threads = npt == 1 ? 512 : npt == 2 ? 1024 : 768;
    // cluster size of the launch: the size the members ask for (HB_RUN_STREAM_CLUSTER, the first member's
    // request), else the largest of 4, 3, 2 that leaves the member with the most work at least 100 nodes
    // per CTA, else one CTA per point. (On the uneven MPR grid, 68 / 84 / 164 / 400 nodes: 4 gives 5.80e9
    // node-steps/s against 5.23e9 for one CTA per point; 6 CTAs, 67 nodes each, 4.77e9.) Members with
    // at least 100 nodes per CTA at that size run each point split over a cluster (their histories in
    // flight shrink by the cluster size); the others run one point per CTA, cluster-size points per item.
    int Cq = 1;
    {
        static const int code_to_c[8] = {0, 1, 2, 4, 8, 3, 5, 6};
        const int v = (int)((members[0].run_flags >> 4) & 0x7);
        if (v) Cq = code_to_c[v];
        else {
            int big = 0;
            for (int i = 1; i < n; i++)
                if ((double)members[i].engine->subs[0].nm * members[i].engine->B * members[i].n_steps >
                    (double)members[big].engine->subs[0].nm * members[big].engine->B * members[big].n_steps)
                    big = i;
            const int nmb = members[big].engine->subs[0].nm;
            for (int c = 4; c >= 2 && Cq == 1; c--)
                if (nmb / c >= 100) Cq = c;
        }
        if (Cq > 1) {
            const int cap = npt == 1 ? hb_stream_queue_grid_1(threads, 48 * 1024, Cq)
                          : npt == 2 ? hb_stream_queue_grid_2(threads, 48 * 1024, Cq) : hb_stream_queue_grid_4(threads, 48 * 1024, Cq);
            if (cap <= 0) return fail(HB_ERR_UNSUPPORTED, "grouped launch: no cluster of %d CTAs fits the device", Cq);
        }
    }
    std::unique_ptr<hb_group> g(new hb_group());
    if (cuda_stream) g->user = (cudaStream_t)cuda_stream;
    else CUDA_TRY(cudaStreamCreateWithFlags(&g->own, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&g->ev0));
    CUDA_TRY(cudaEventCreate(&g->ev1));
    g->m.resize(n);
    size_t smem = 0;
    for (int i = 0; i < n; i++) {
        const hb_group_member& mb = members[i];
        hb_group::Member& gm = g->m[i];
        hb_engine* e = gm.e = mb.engine;
        hb_status s = validate_noise(e, mb.noise, mb.noise_len, mb.n_steps);
        if (s) return s;
        hb_sweep_point dim{mb.sub_idx, mb.param_idx, mb.values, mb.n_values};
        if ((s = build_tables(e, &dim, 1, false, gm.T))) return s;
        if ((s = reset_state(e))) return s;
        e->bold_removed = false;
        if ((s = reset_bold_device(e))) return s;
        const float* noise_dev = nullptr;
        if (mb.noise && mb.noise_len > 0) {
            CUDA_TRY(gm.noise.ensure((size_t)mb.noise_len));
            CUDA_TRY(cudaMemcpy(gm.noise.p, mb.noise, (size_t)mb.noise_len * 4, cudaMemcpyHostToDevice));
            noise_dev = gm.noise.p;
        }
        // a member with at least 100 nodes per CTA at the launch's cluster size runs its points split over
        // a cluster; the others one point per CTA
        const int mc = (Cq > 1 && e->subs[0].nm / Cq >= 100) ? Cq : 1;
        const uint32_t flags = (mb.run_flags & ~(uint32_t)(0x7u << 24) & ~(uint32_t)(0x7u << 4)) | HB_RUN_STREAM |
                               HB_RUN_STREAM_NPT(npt) | HB_RUN_STREAM_CLUSTER(mc);
        if ((s = run_setup(e, gm.T, mb.n_steps, flags, nullptr, noise_dev ? noise_dev : e->x0.p, nullptr, gm.P))) return s;
        if (gm.P.stream_npt != npt)
            return fail(HB_ERR_UNSUPPORTED, "member %d cannot run in the streamed-history kernel (one subnetwork, one sparse "
                        "projection with per-edge delays >= %d steps)", i, 2 * HB_STREAM_K - 1);
        if (e->kernel_model < 0 || (gm.P.fast == 1 && e->subs[0].ncvar != 1))
            return fail(HB_ERR_UNSUPPORTED, "member %d: no streamed-history kernel path for its model and coupling", i);
        smem = std::max(smem, gm.P.stream_smem);
        gm.P.a.s0 = 0;
        gm.P.a.n_steps = (int)mb.n_steps;
        gm.P.a.load_ring = 0;
        gm.P.a.store_ring = 1;
        gm.P.a.traj = nullptr;
        if (gm.P.any_stoch) gm.P.a.noise = noise_dev;
        // Balloon-Windkessel start state for the graph's reset
        gm.bw_init.resize(e->bold.size());
        for (size_t k = 0; k < e->bold.size(); k++) {
            const size_t words = 5 * (size_t)((e->flags & HB_SEM_BOLD_PER_POINT) ? e->B : 1) * e->subs[0].nnodes;
            CUDA_TRY(gm.bw_init[k].ensure(words));
            CUDA_TRY(cudaMemcpyAsync(gm.bw_init[k].p, e->bold[k].bw.p, words * 4, cudaMemcpyDeviceToDevice, e->stream()));
        }
        for (int mo = 0; mo < gm.P.n_bold_active && !gm.P.bold_pp; mo++) {
            int n_win = gm.P.a.bold.n_full[mo] + (gm.P.a.bold.partial[mo] > 0 ? 1 : 0);
            CUDA_TRY(e->means.ensure((size_t)std::max(n_win, 1) * gm.P.N0));
        }
        CUDA_TRY(cudaStreamSynchronize(e->stream()));
    }
    const int budget = npt == 1 ? hb_stream_queue_budget_1() : npt == 2 ? hb_stream_queue_budget_2() : hb_stream_queue_budget_4();
    if (budget < 0 || smem + 64 > (size_t)budget) return fail(HB_ERR_UNSUPPORTED, "grouped launch: shared memory budget exceeded");
    // jobs, longest work per CTA first; a split member's item is one point over a cluster, another
    // member's item is Cq points, one per CTA
    auto is_split = [&](int i) { return Cq > 1 && g->m[i].P.a.stream_cluster == Cq; };
    auto work = [&](int i) {
        return (double)g->m[i].e->subs[0].nm * members[i].n_steps / (is_split(i) ? Cq : 1);
    };
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work(x) > work(y); });
    std::vector<StreamJob> jobs(n);
    int blocks = 0;
    for (int k = 0; k < n; k++) {
        hb_group::Member& gm = g->m[order[k]];
        const bool sp = is_split(order[k]);
        jobs[k].net = gm.e->d_net;
        jobs[k].args = gm.P.a;
        jobs[k].first_block = blocks;
        jobs[k].n_points = gm.e->B;
        jobs[k].model = gm.e->kernel_model;
        jobs[k].pre = gm.P.fast;
        jobs[k].split = sp ? 1 : 0;
        blocks += sp ? gm.e->B : (gm.e->B + Cq - 1) / Cq;
    }
    CUDA_TRY(g->jobs.ensure(n));
    CUDA_TRY(g->counter.ensure(1));
    CUDA_TRY(cudaMemcpy(g->jobs.p, jobs.data(), n * sizeof(StreamJob), cudaMemcpyHostToDevice));
    const int grid = npt == 1 ? hb_stream_queue_grid_1(threads, smem, Cq) : npt == 2 ? hb_stream_queue_grid_2(threads, smem, Cq)
                                                                          : hb_stream_queue_grid_4(threads, smem, Cq);
    if (grid < 1) return fail(HB_ERR_CUDA, "grouped launch: cannot size the work-queue grid");
    // the whole run as one graph: member resets, the queue counter, the grouped launch, batch-mean BOLD reductions
    cudaStream_t st = g->stream();
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaSuccess;
    for (auto& gm : g->m) {
        hb_engine* e = gm.e;
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(e->state.p, e->x0.p, (size_t)e->B * e->state_len * 4, cudaMemcpyDeviceToDevice, st);
        if (ce == cudaSuccess) ce = cudaMemsetAsync(e->flags_buf.p, 0, 2 * sizeof(int), st);
        for (size_t k = 0; k < gm.bw_init.size() && ce == cudaSuccess; k++)
            ce = cudaMemcpyAsync(e->bold[k].bw.p, gm.bw_init[k].p, gm.bw_init[k].n * 4, cudaMemcpyDeviceToDevice, st);
    }
    // external event records become nodes of the graph, so the replay times the launch itself
    if (ce == cudaSuccess) ce = cudaMemsetAsync(g->counter.p, 0, sizeof(int), st);
    if (ce == cudaSuccess) ce = cudaEventRecordWithFlags(g->ev0, st, cudaEventRecordExternal);
    if (ce == cudaSuccess)
        ce = npt == 1 ? hb_launch_stream_queue_1(g->jobs.p, n, blocks, g->counter.p, grid, threads, smem, Cq, st)
           : npt == 2 ? hb_launch_stream_queue_2(g->jobs.p, n, blocks, g->counter.p, grid, threads, smem, Cq, st)
                      : hb_launch_stream_queue_4(g->jobs.p, n, blocks, g->counter.p, grid, threads, smem, Cq, st);
    if (ce == cudaSuccess) ce = cudaEventRecordWithFlags(g->ev1, st, cudaEventRecordExternal);
    for (auto& gm : g->m) {
        for (int mo = 0; mo < gm.P.n_bold_active && !gm.P.bold_pp && ce == cudaSuccess; mo++) {
            int n_win = gm.P.a.bold.n_full[mo] + (gm.P.a.bold.partial[mo] > 0 ? 1 : 0);
            ce = hb_launch_bold_batch_mean(gm.P.a.bold, mo, n_win, gm.e->B, gm.e->means.p, st);
        }
    }
    cudaError_t ce2 = cudaStreamEndCapture(st, &g->graph);
    if (ce != cudaSuccess) return fail(HB_ERR_CUDA, "capturing the grouped launch: %s", cudaGetErrorString(ce));
    if (ce2 != cudaSuccess) return fail(HB_ERR_CUDA, "capturing the grouped launch: %s", cudaGetErrorString(ce2));
    CUDA_TRY(cudaGraphInstantiate(&g->exec, g->graph, 0));
    for (auto& gm : g->m) gm.e->last_kind = 5;
    *out = g.release();
    return HB_OK;
}

hb_status hb_group_execute(hb_group* g) {
    if (!g || !g->exec) return fail(HB_ERR_INVALID_STATE, "group not prepared");
    for (auto& gm : g->m) {
        hb_engine* e = gm.e;
        e->step = 0;
        e->bold_removed = false;
        for (auto& bh : e->bold) { bh.times.clear(); bh.n_out = 0; bh.out.clear(); }
    }
    CUDA_TRY(cudaGraphLaunch(g->exec, g->stream()));
    CUDA_TRY(cudaStreamSynchronize(g->stream()));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
    g->last_ms = ms;
    for (auto& gm : g->m) {
        hb_result sink;  // run_finish copies the BOLD outputs of the run when given a result
        hb_status s = run_finish(gm.e, gm.P, &sink, false);
        gm.e->last_ms = ms;
        gm.e->last_launches = 1;
        if (s) return s;
    }
    g->executed = true;
    return HB_OK;
}

hb_status hb_group_result(hb_group* g, int32_t i, hb_result** out) {
    if (!g || !out) return fail(HB_ERR_INVALID_STATE, "NULL argument");
    *out = nullptr;
    if (i < 0 || i >= (int)g->m.size()) return fail(HB_ERR_INVALID_STATE, "member %d out of range", i);
    if (!g->executed) return fail(HB_ERR_INVALID_STATE, "group not executed");
    hb_group::Member& gm = g->m[i];
    hb_result* r = new hb_result();
    hb_status s = collect(gm.e, gm.P.n_steps, r);
    if (s) { delete r; return s; }
    r->elapsed_ms = g->last_ms;
    r->params = gm.T.param_values;
    r->has_traj = false;
    *out = r;
    return HB_OK;
}

hb_status hb_group_last_kernel_time(const hb_group* g, double* ms) {
    if (!g || !ms) return fail(HB_ERR_INVALID_STATE, "NULL argument");
    *ms = g->last_ms;
    return HB_OK;
}

void hb_group_destroy(hb_group* g) { delete g; }

// ======================================================================================
// Adjoint of a functional-connectivity loss (no counterpart in the reference)
// ======================================================================================

struct AdjWorkspace {
    DBuf<int> cptr, ctgt, cdel;
    DBuf<float> cw, Y, S, ck_state, ck_ring, scratch, mu_ring, lam, target, mean, sdev, coef, rk, M, fc;
    DBuf<double> loss, gG, gA, gB, ga, moments;
};

hb_status hb_engine_adjoint_fc(hb_engine* e, const float* gain_values, int32_t n_values, int64_t n_steps,
                               const float* target_fc, int32_t checkpoint_every, hb_adjoint_out* out) {
    if (!e || !gain_values || !target_fc || !out) return fail(HB_ERR_INVALID_STATE, "NULL argument");
    if (n_values != e->B) return fail(HB_ERR_INVALID_STATE, "expected %d gain values, got %d", e->B, n_values);
    if (n_steps < 2 || n_steps > (1 << 30)) return fail(HB_ERR_INVALID_STATE, "n_steps must be in [2, 2^30]");
    if (e->subs.size() != 1 || e->projs.size() != 1 || e->subs[0].model != HBM_JR || e->subs[0].nmodes != 1)
        return fail(HB_ERR_UNSUPPORTED, "the FC adjoint needs one JansenRit subnetwork (one mode) and one projection");
    if (!e->subs[0].node_params.empty())
        return fail(HB_ERR_UNSUPPORTED, "the FC adjoint differentiates one JansenRit parameter row per point (no node_params)");
    HostProj& hp = e->projs[0];
    if (hp.kind != W_SPARSE || hp.dmode != HBD_EDGE)
        return fail(HB_ERR_UNSUPPORTED, "the FC adjoint needs a CSR projection with per-edge delays (HB_SEM_DELAY_RING)");
    if (hp.cf.kind != HBC_SIGMOIDAL && hp.cf.kind != HBC_LINEAR)
        return fail(HB_ERR_UNSUPPORTED, "the FC adjoint supports Sigmoidal and Linear coupling");
    if (hp.ncv != 1 || !hp.direct) return fail(HB_ERR_UNSUPPORTED, "the FC adjoint needs the coupling from and into the first coupling variable");
    const int adj_integ = eff_integrator(e, HBM_JR);
    if (adj_integ != HBI_HEUN_DET && adj_integ != HBI_RK4)
        return fail(HB_ERR_UNSUPPORTED, "the FC adjoint differentiates deterministic Heun or RK4");
    const int N = e->subs[0].nm, B = e->B;
    if (N > 120) return fail(HB_ERR_UNSUPPORTED, "the FC adjoint supports up to 120 nodes");
    int dmin = 1 << 30;
    for (uint32_t m : hp.edges) dmin = std::min(dmin, (int)(m >> 16));
    if (hp.edges.empty()) dmin = 8;
    if (dmin < 1) return fail(HB_ERR_UNSUPPORTED, "the FC adjoint needs every edge delay >= 1");
    const int K = std::min(dmin, 8);
    const int R = hp.maxd + 2 * K + 1;
    int dev = 0, optin = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if ((size_t)R * N * 4 + 2 * ((size_t)(N + 1) * 4 + hp.edges.size() * 8) + (size_t)K * N * 4 + 1024 > (size_t)optin)
        return fail(HB_ERR_UNSUPPORTED, "the delay ring and edge tables of one point do not fit shared memory");
    int CK = std::max(K, (checkpoint_every + K - 1) / K * K);
    const int T = (int)n_steps;
    // checkpoint_every <= 0: keep x(s), g(s) of every step when that takes at most a quarter of the
    // free device memory (no re-computation in the reverse sweep); else checkpoint every 500 steps
    int store_all = 0;
    if (checkpoint_every <= 0) {
        size_t free_b = 0, total_b = 0;
        CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
        const double need = (double)T * B * N * 8 * 4 + 2.0 * T * B * N * 4;
        if (need <= 0.25 * (double)free_b) { store_all = 1; CK = ((T + K - 1) / K) * K; }
        else CK = (500 + K - 1) / K * K;
    }
    const int n_ck = (T + CK - 1) / CK;
    // tables of the gain sweep (Sigmoidal a = parameter 3, Linear a = parameter 0)
    const int gain_param = hp.cf.kind == HBC_SIGMOIDAL ? 3 : 0;
    hb_sweep_point dim{-1, gain_param, gain_values, n_values};
    RunTables Tb;
    hb_status s = build_tables(e, &dim, 1, false, Tb);
    if (s) return s;
    if ((s = upload_net(e, Tb))) return s;
    if ((s = reset_state(e))) return s;
    // out-edges of every source node (transpose of the CSR rows)
    std::vector<int> cptr(N + 1, 0), ctgt(hp.edges.size()), cdel(hp.edges.size());
    std::vector<float> cw(hp.edges.size());
    for (uint32_t m : hp.edges) cptr[(m & 0xffffu) + 1]++;
    for (int j = 0; j < N; j++) cptr[j + 1] += cptr[j];
    {
        std::vector<int> fill(cptr.begin(), cptr.end() - 1);
        for (int i = 0; i < N; i++)
            for (int k = hp.rowptr[i]; k < hp.rowptr[i + 1]; k++) {
                const int src = (int)(hp.edges[k] & 0xffffu), q = fill[src]++;
                ctgt[q] = i; cdel[q] = (int)(hp.edges[k] >> 16); cw[q] = hp.ew[k];
            }
    }
    std::unique_ptr<AdjWorkspace> W(new AdjWorkspace());
    cudaStream_t st = e->stream();
    const size_t nnz = std::max<size_t>(hp.edges.size(), 1);
    CUDA_TRY(W->cptr.ensure(N + 1)); CUDA_TRY(W->ctgt.ensure(nnz)); CUDA_TRY(W->cdel.ensure(nnz)); CUDA_TRY(W->cw.ensure(nnz));
    CUDA_TRY(cudaMemcpyAsync(W->cptr.p, cptr.data(), (N + 1) * 4, cudaMemcpyHostToDevice, st));
    if (!hp.edges.empty()) {
        CUDA_TRY(cudaMemcpyAsync(W->ctgt.p, ctgt.data(), ctgt.size() * 4, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(W->cdel.p, cdel.data(), cdel.size() * 4, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(W->cw.p, cw.data(), cw.size() * 4, cudaMemcpyHostToDevice, st));
    }
    const size_t TBN = (size_t)T * B * N;
    CUDA_TRY(W->Y.ensure(TBN)); CUDA_TRY(W->S.ensure(TBN));
    CUDA_TRY(W->ck_state.ensure(store_all ? 1 : (size_t)n_ck * B * N * 6));
    CUDA_TRY(W->ck_ring.ensure(store_all ? 1 : (size_t)n_ck * B * R * N));
    // the re-computation of one segment overlaps the reverse of the next: two segment buffers
    CUDA_TRY(W->scratch.ensure((size_t)B * CK * N * 8 * (store_all ? 1 : 2)));
    CUDA_TRY(W->lam.ensure((size_t)B * N * 6));
    CUDA_TRY(W->mu_ring.ensure((size_t)B * R * N));
    CUDA_TRY(W->target.ensure((size_t)N * N));
    CUDA_TRY(cudaMemcpyAsync(W->target.p, target_fc, (size_t)N * N * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(W->mean.ensure((size_t)B * N)); CUDA_TRY(W->sdev.ensure((size_t)B * N)); CUDA_TRY(W->coef.ensure((size_t)B * N));
    CUDA_TRY(W->rk.ensure((size_t)B * N)); CUDA_TRY(W->M.ensure((size_t)B * N * N)); CUDA_TRY(W->fc.ensure((size_t)B * N * N));
    CUDA_TRY(W->loss.ensure(B)); CUDA_TRY(W->gG.ensure(B));
    CUDA_TRY(W->gA.ensure((size_t)B * N)); CUDA_TRY(W->gB.ensure((size_t)B * N)); CUDA_TRY(W->ga.ensure((size_t)B * N));
    {
        const size_t Wn = (size_t)(N + 3) / 4 * 4;
        CUDA_TRY(W->moments.ensure((size_t)B * hb_adjoint_moment_slices(B, T) * (Wn * Wn + Wn)));
    }
    HbAdjointLaunch L;
    L.B = B; L.N = N; L.T = T; L.R = R; L.K = K; L.CK = CK; L.n_ck = n_ck; L.nnz = (int)hp.edges.size();
    L.store_all = store_all;
    L.cfk = hp.cf.kind; L.gain_idx = gain_param;
    L.dt = e->net.dt; L.dt_half = e->net.dt_half;
    L.rk4 = adj_integ == HBI_RK4 ? 1 : 0; L.dt_h2 = e->net.dt_h2; L.dt_sixth = e->net.dt_sixth;
    L.x0 = e->x0.p; L.rowptr = hp.d_rowptr; L.edges = hp.d_edges; L.ew = hp.d_ew;
    L.cptr = W->cptr.p; L.ctgt = W->ctgt.p; L.cdel = W->cdel.p; L.cw = W->cw.p;
    L.Y = W->Y.p; L.S = W->S.p; L.ck_state = W->ck_state.p; L.ck_ring = W->ck_ring.p; L.scratch = W->scratch.p;
    L.mu_ring = W->mu_ring.p; L.target = W->target.p; L.mean = W->mean.p; L.sdev = W->sdev.p; L.coef = W->coef.p;
    L.rk = W->rk.p; L.M = W->M.p; L.fc = W->fc.p; L.loss = W->loss.p; L.gG = W->gG.p; L.gA = W->gA.p; L.gB = W->gB.p;
    L.ga = W->ga.p;
    L.moments = W->moments.p;
    L.slices = hb_adjoint_moment_slices(B, T);
    L.pipelined = dmin >= 2 * K - 1 ? 1 : 0;
    L.lam_g = W->lam.p;
    L.dmin = dmin;
    cudaEvent_t ev[4];
    for (auto& v : ev) CUDA_TRY(cudaEventCreate(&v));
    cudaError_t ce = cudaEventRecord(ev[0], st);
    if (ce == cudaSuccess) ce = hb_launch_adjoint(e->d_net, L, 0, st);
    if (ce == cudaSuccess) ce = cudaEventRecord(ev[1], st);
    if (ce == cudaSuccess) ce = hb_launch_adjoint(e->d_net, L, 1, st);
    if (ce == cudaSuccess) ce = cudaEventRecord(ev[2], st);
    if (ce == cudaSuccess) ce = hb_launch_adjoint(e->d_net, L, 2, st);
    if (ce == cudaSuccess) ce = cudaEventRecord(ev[3], st);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(ev[3]);
    float ms[3] = {0, 0, 0};
    for (int k = 0; k < 3 && ce == cudaSuccess; k++) ce = cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]);
    for (auto& v : ev) cudaEventDestroy(v);
    if (ce != cudaSuccess) return fail(HB_ERR_CUDA, "adjoint: %s", cudaGetErrorString(ce));
    e->last_ms = (double)ms[0] + ms[1] + ms[2];
    e->last_launches = 5;
    e->last_kind = 6;
    out->forward_ms = ms[0];
    out->statistics_ms = ms[1];
    out->reverse_ms = ms[2];
    if (out->loss) CUDA_TRY(cudaMemcpy(out->loss, W->loss.p, B * 8, cudaMemcpyDeviceToHost));
    if (out->d_gain) CUDA_TRY(cudaMemcpy(out->d_gain, W->gG.p, B * 8, cudaMemcpyDeviceToHost));
    if (out->d_A) CUDA_TRY(cudaMemcpy(out->d_A, W->gA.p, (size_t)B * N * 8, cudaMemcpyDeviceToHost));
    if (out->d_B) CUDA_TRY(cudaMemcpy(out->d_B, W->gB.p, (size_t)B * N * 8, cudaMemcpyDeviceToHost));
    if (out->d_a) CUDA_TRY(cudaMemcpy(out->d_a, W->ga.p, (size_t)B * N * 8, cudaMemcpyDeviceToHost));
    if (out->fc) CUDA_TRY(cudaMemcpy(out->fc, W->fc.p, (size_t)B * N * N * 4, cudaMemcpyDeviceToHost));
    if (out->y) CUDA_TRY(cudaMemcpy(out->y, W->Y.p, TBN * 4, cudaMemcpyDeviceToHost));
    for (auto* b : {&W->Y, &W->S, &W->ck_state, &W->ck_ring, &W->scratch, &W->mu_ring, &W->lam, &W->target, &W->mean, &W->sdev,
                    &W->coef, &W->rk, &W->M, &W->fc, &W->cw})
        b->release();
    W->cptr.release(); W->ctgt.release(); W->cdel.release();
    W->loss.release(); W->gG.release(); W->gA.release(); W->gB.release(); W->ga.release(); W->moments.release();
    return HB_OK;
}
