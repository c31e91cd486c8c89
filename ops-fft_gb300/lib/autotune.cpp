// autotune.cpp - timed choice of the planner's options for a made plan.
//
// The planner picks, per length, the first specialised row kernel
// (codelet_list.h), its transform groups per CTA and prefetch stages from a
// residency score, and the first cluster configuration (cluster_list.h),
// with clusters used for 4096-point transforms only at small batches.  The
// tuner builds the plan once per candidate set of choices, keeps the ones
// whose launches differ, times each on scratch buffers of the plan's shape
// (the batch capped at 256 MB of input), and re-plans with the fastest;
// the planner's own choice is kept unless another is at least 2 % faster.
// Choices are cached per (device, kind, length, batch, layout) for the
// process and, when OPS_FFT_PLAN_TUNE_CACHE names a file, across processes
// (one line per key; a line that does not parse is ignored, so a damaged
// file only costs a re-tune).
//
// The reference has no tuner: its radix choices are fixed tables
// (src/common/host/fft_exec_helper.h:76-139).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "handle.h"

namespace gfft {
namespace {

std::mutex g_mu;
std::map<std::string, PlanHints> g_cache;
bool g_file_loaded = false;

const char* cache_path()
{
    const char* p = std::getenv("OPS_FFT_PLAN_TUNE_CACHE");
    return (p && *p) ? p : nullptr;
}

// file lines: "<key> <variant> <ng> <nst> <codelets> <cluster> <cluster_c> <pp>"
void load_file()
{
    if (g_file_loaded) return;
    g_file_loaded = true;
    const char* path = cache_path();
    if (!path) return;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string key;
        PlanHints h;
        if (!(is >> key >> h.codelet_variant >> h.codelet_ng >> h.codelet_nst >> h.codelets >> h.cluster >>
              h.cluster_c >> h.codelet_pp))
            continue;
        if (h.codelet_variant < -1 || h.codelet_variant > 64 || h.codelet_ng < 0 || h.codelet_ng > 15 ||
            h.codelet_nst < 0 || h.codelet_nst > 4 || h.codelets < -1 || h.codelets > 1 || h.cluster < -1 ||
            h.cluster > 1 || (h.cluster_c != 0 && h.cluster_c != 2 && h.cluster_c != 4 && h.cluster_c != 8 &&
                              h.cluster_c != 16) ||
            h.codelet_pp < -1 || h.codelet_pp > 1)
            continue;
        g_cache[key] = h;
    }
}

void save_file()
{
    const char* path = cache_path();
    if (!path) return;
    std::ofstream f(path, std::ios::trunc);
    for (const auto& kv : g_cache) {
        const PlanHints& h = kv.second;
        f << kv.first << ' ' << h.codelet_variant << ' ' << h.codelet_ng << ' ' << h.codelet_nst << ' ' << h.codelets
          << ' ' << h.cluster << ' ' << h.cluster_c << ' ' << h.codelet_pp << '\n';
    }
}

std::string cache_key(const aclfftHandle_t* h)
{
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        prop.multiProcessorCount = 0;
        prop.name[0] = 0;
    }
    std::string name = prop.name;
    for (char& c : name)
        if (c == ' ') c = '_';
    std::ostringstream os;
    os << name << ':' << prop.multiProcessorCount << ':' << (int)h->type << ':' << h->rank << ':' << h->lengths[0]
       << ':' << (h->rank >= 2 ? h->lengths[1] : 1) << ':' << (h->rank == 3 ? h->lengths[2] : 1) << ':' << h->batch
       << ':' << h->stride[0] << ':' << h->precision;
    return os.str();
}

// What distinguishes two plans' launches: kernel family, specialised build,
// CTA shape and the on-chip radices of every step of the primary list.
std::string signature(const StepList& sl)
{
    std::ostringstream os;
    for (const Step& s : sl.steps) {
        os << (int)s.kind << '/';
        switch (s.kind) {
        case Step::ROW:
            os << s.row.codelet << ',' << s.row.ngroups << ',' << s.row.nstage << ',' << s.row.nbuf << ','
               << s.row.tfpc << ',';
            for (int p = 0; p < s.row.ip.npass; ++p) os << s.row.ip.pass[p].radix << '.';
            break;
        case Step::COL:
            os << s.col.codelet << ',' << s.col.tfpc << ',';
            for (int p = 0; p < s.col.ip.npass; ++p) os << s.col.ip.pass[p].radix << '.';
            break;
        case Step::CLUSTER: os << s.cl.kid << ',' << s.cl.csize; break;
        default: break;
        }
        os << ';';
    }
    return os.str();
}

// The candidate choices: the planner's own, every other specialised build
// of the length, other group/stage/work-buffer shapes of the codelet, cluster sizes,
// clusters forced on or off, and no codelets at all.
std::vector<PlanHints> candidates()
{
    std::vector<PlanHints> c;
    c.push_back(PlanHints{});
    for (int v = 1; v <= 5; ++v) {
        PlanHints h;
        h.codelet_variant = v;
        c.push_back(h);
    }
    for (int pp : {0, 1})
        for (int nst : {2, 3})
            for (int ng : {1, 2, 4, 8}) {
                PlanHints h;
                h.codelet_ng = ng;
                h.codelet_nst = nst;
                h.codelet_pp = pp;
                c.push_back(h);
            }
    for (int cc : {4, 8, 16}) {
        PlanHints h;
        h.cluster_c = cc;
        c.push_back(h);
    }
    {
        PlanHints h;
        h.cluster = 0;
        c.push_back(h);
        h.cluster = 1;
        c.push_back(h);
    }
    {
        PlanHints h;
        h.codelets = 0;
        c.push_back(h);
    }
    return c;
}

struct Scratch {
    void* in = nullptr;
    void* out = nullptr;
    size_t bytes = 0;
    ~Scratch()
    {
        if (in) cudaFree(in);
        if (out) cudaFree(out);
    }
};

// Median time of `reps` timed launches of the primary list (after two
// untimed ones) on `st`; negative on failure.
float time_impl(PlanImpl* impl, Scratch& sc, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, int reps)
{
    for (int i = 0; i < 2; ++i)
        if (launch_primary(impl, sc.in, sc.out, st) != 0) return -1.f;
    std::vector<float> ts;
    for (int i = 0; i < reps; ++i) {
        if (cudaEventRecord(e0, st) != cudaSuccess || launch_primary(impl, sc.in, sc.out, st) != 0 ||
            cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
            return -1.f;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ts.push_back(ms);
    }
    std::sort(ts.begin(), ts.end());
    return ts[ts.size() / 2];
}

}  // namespace

aclfftResult autotune_plan(aclfftHandle_t* h)
{
    if (!h->is_initialized || !h->impl) return ACLFFT_INVALID_PLAN;
    PlanImpl* cur = h->impl;
    if (!cur->device_ready) {
        if (plan_device_setup(cur) != ACLFFT_SUCCESS || !cur->device_ready) return ACLFFT_EXEC_FAILED;
    }
    // split-precision forms have fixed launches; VERTICAL plans one column
    // kernel; double precision one pass kernel per radix
    if (h->precision != 0 || (h->rank == 1 && h->stride[0] > 1) || !cur->lists[0].supported || cur->prob.dbl) {
        h->tuned = 0;
        h->tune_candidates = 0;
        return ACLFFT_SUCCESS;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    load_file();
    const std::string key = cache_key(h);
    auto hit = g_cache.find(key);
    if (hit != g_cache.end()) {
        if (!(hit->second == h->hints)) {
            const PlanHints old = h->hints;
            h->hints = hit->second;
            if (replan(h) != ACLFFT_SUCCESS) {
                h->hints = old;
                return ACLFFT_EXEC_FAILED;
            }
        }
        h->tuned = 1;
        h->tune_candidates = 0;
        return ACLFFT_SUCCESS;
    }

    // trial problem: the plan's shape with the batch capped at 256 MB of input
    aclfftHandle_t trial;
    trial.rank = h->rank;
    std::memcpy(trial.lengths, h->lengths, sizeof trial.lengths);
    std::memcpy(trial.stride, h->stride, sizeof trial.stride);
    trial.type = h->type;
    trial.precision = h->precision;
    int64_t pts = 1;
    for (int a = 0; a < h->rank; ++a) pts *= h->lengths[a];
    const int64_t last = h->lengths[h->rank - 1];
    const int64_t half = pts / last * (last / 2 + 1);  // bins of one half spectrum
    const int64_t in_per = h->type == ACLFFT_C2C ? pts * 8 : (h->type == ACLFFT_R2C ? pts * 4 : half * 8);
    const int64_t out_per = h->type == ACLFFT_C2C ? pts * 8 : (h->type == ACLFFT_R2C ? half * 8 : pts * 4);
    const int64_t cap = std::max<int64_t>(1, ((int64_t)256 << 20) / std::max<int64_t>(in_per, 1));
    trial.batch = (int32_t)std::min<int64_t>(h->batch, cap);
    const int64_t in_bytes = in_per * trial.batch;
    const int64_t out_bytes = (h->type == ACLFFT_C2R ? out_per : std::max(in_per, out_per)) * trial.batch;

    Scratch sc;
    sc.bytes = (size_t)std::max(in_bytes, out_bytes);
    if (dev_alloc(&sc.in, sc.bytes) != cudaSuccess || dev_alloc(&sc.out, sc.bytes) != cudaSuccess ||
        cudaMemset(sc.in, 0, sc.bytes) != cudaSuccess) {
        cudaGetLastError();
        set_last_error("autotune: scratch allocation failed");
        return ACLFFT_ALLOC_FAILED;
    }
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        if (st) cudaStreamDestroy(st);
        if (e0) cudaEventDestroy(e0);
        return ACLFFT_EXEC_FAILED;
    }
    std::vector<std::string> seen;
    float best_t = -1.f, base_t = -1.f;
    PlanHints best;
    int timed = 0;
    for (const PlanHints& cand : candidates()) {
        trial.hints = cand;
        aclfftResult why = ACLFFT_SUCCESS;
        PlanImpl* impl = plan_steps(&trial, &why);
        if (!impl) continue;
        const std::string sig = signature(impl->lists[0]);
        const bool dup = std::find(seen.begin(), seen.end(), sig) != seen.end();
        if (dup || !impl->lists[0].supported || plan_device_setup(impl) != ACLFFT_SUCCESS || !impl->device_ready) {
            cudaGetLastError();
            plan_impl_free(impl);
            delete impl;
            continue;
        }
        seen.push_back(sig);
        const float t = time_impl(impl, sc, st, e0, e1, 5);
        plan_impl_free(impl);
        delete impl;
        if (t < 0.f) {
            cudaGetLastError();
            continue;
        }
        ++timed;
        if (cand == PlanHints{}) base_t = t;
        if (best_t < 0.f || t < best_t) {
            best_t = t;
            best = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (best_t < 0.f) {
        set_last_error("autotune: no candidate ran");
        return ACLFFT_EXEC_FAILED;
    }
    // keep the planner's choice unless another is clearly faster
    if (base_t > 0.f && best_t > 0.98f * base_t) best = PlanHints{};
    g_cache[key] = best;
    save_file();
    const PlanHints old = h->hints;
    if (!(best == h->hints)) {
        h->hints = best;
        if (replan(h) != ACLFFT_SUCCESS) {
            h->hints = old;
            return ACLFFT_EXEC_FAILED;
        }
    }
    h->tuned = 1;
    h->tune_candidates = timed;
    return ACLFFT_SUCCESS;
}

}  // namespace gfft

extern "C" {

ACLFFT_API aclfftResult aclfftSetAutotune(aclfftHandle plan, int mode)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_PARAM(mode == 0 || mode == 1, ACLFFT_INVALID_VALUE);
    plan->autotune = mode;
    if (mode == 1 && plan->is_initialized && plan->impl) return gfft::autotune_plan(plan);
    return ACLFFT_SUCCESS;
}

}  // extern "C"
