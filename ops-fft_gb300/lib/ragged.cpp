// ragged.cpp - ragged batches: many 1D transforms of different lengths and
// kinds executed by one persistent launch (aclfftRagged* extension).
//
// Plan creation groups the transforms into classes (kind, length), builds
// each class's on-chip plan - one Stockham transform, or a two-step split
// L = L1 * L2 for lengths beyond one CTA - and the work-item table the
// persistent kernel consumes (csrc/ragged.cu).  Item order: the first steps
// of long transforms, then the on-chip groups by decreasing cost (longest
// first, so the tail of the launch is short items), then the second steps
// and post-processes, which wait on counters for the earlier steps.
//
// Autotuning: per class, candidate radix orders and thread counts are timed
// in isolation on scratch buffers and the fastest is kept; choices are
// cached process-wide (and in a text file when OPS_FFT_TUNE_CACHE names
// one) keyed by (kind, length).
//
// Execution: a counter reset and the kernel launch, captured once per
// (input, output, direction) into a CUDA graph on a plan-owned stream and
// replayed on the caller's stream; when the caller's stream is itself being
// captured, the two operations are issued directly into that capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <new>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include "handle.h"

namespace {

using namespace gfft;

constexpr int kThreads = 256;
constexpr int kSmemBudget = 110 * 1024;  // per CTA (two CTAs per SM)
constexpr int kMaxTwWindow = 5120;       // float2 entries of a pass-table window staged in shared memory
constexpr int kMaxSingle = 4096;         // longest on-chip complex length
constexpr int64_t kMaxLength = 1 << 24;

int spad_h(int i) { return i + (i >> 4); }
int row_pitch(int L) { return spad_h(L - 1) + 2; }

struct Variant {
    std::vector<int> rad;
    int nthr = 0;
};

bool primes_le_13(int64_t n)
{
    for (int p : {2, 3, 5, 7, 11, 13})
        while (n % p == 0) n /= p;
    return n == 1;
}

int nthr_for(int L, const std::vector<int>& rad, int cap)
{
    int nbf = 1;
    for (int r : rad) nbf = std::max(nbf, L / r);
    if (nbf <= cap) return nbf;
    const int waves = (nbf + cap - 1) / cap;
    return (nbf + waves - 1) / waves;
}

// Candidate on-chip plans of length L: the planner's radix choice, its
// reverse, a radix <= 8 factorisation, each with the natural thread count
// and half of it (two butterflies per thread and pass).
std::vector<Variant> candidates(int L, int cap)
{
    std::vector<std::vector<int>> rads;
    std::vector<int> base = choose_radices(L);
    if (base.empty()) return {};
    rads.push_back(base);
    std::vector<int> rev(base.rbegin(), base.rend());
    if (rev != base) rads.push_back(rev);
    {
        std::vector<int> small;
        int rem = L;
        for (int r : {8, 4, 2, 7, 5, 3, 13, 11})
            while (rem % r == 0 && (int)small.size() < kMaxPass) {
                small.push_back(r);
                rem /= r;
            }
        if (rem == 1 && !small.empty() && small != base && small != rev) rads.push_back(small);
    }
    std::vector<Variant> out;
    for (auto& r : rads) {
        const int t = nthr_for(L, r, cap);
        out.push_back({r, t});
        if (t >= 64 && t % 2 == 0) out.push_back({r, t / 2});
    }
    return out;
}

struct Key {
    int type, n;
    bool operator<(const Key& o) const { return type != o.type ? type < o.type : n < o.n; }
};

// Tuned choice per class: variant indices of the first and second transform.
struct Choice {
    int v1 = 0, v2 = 0;
};

std::mutex g_tune_mu;
std::map<Key, Choice> g_tuned;
bool g_tune_file_loaded = false;

void load_tune_file()
{
    if (g_tune_file_loaded) return;
    g_tune_file_loaded = true;
    const char* path = std::getenv("OPS_FFT_TUNE_CACHE");
    if (!path || !*path) return;
    std::ifstream f(path);
    int t, n, a, b;
    while (f >> t >> n >> a >> b) g_tuned[{t, n}] = {a, b};
}

void save_tune_file()
{
    const char* path = std::getenv("OPS_FFT_TUNE_CACHE");
    if (!path || !*path) return;
    std::ofstream f(path, std::ios::trunc);
    for (auto& kv : g_tuned) f << kv.first.type << ' ' << kv.first.n << ' ' << kv.second.v1 << ' ' << kv.second.v2 << '\n';
}

struct ClassPlan {
    RagClass dev{};
    std::vector<Variant> cand1, cand2;
    std::vector<InnerPlan> ip1, ip2;  // per candidate
    Choice choice;
    bool tuned = false;
    std::vector<int> members;  // transform indices
};

}  // namespace

struct aclfftRaggedPlan_t {
    int count = 0;
    std::vector<int> len, type;
    std::vector<int64_t> in_off, out_off;
    std::vector<ClassPlan> classes;
    std::vector<RagXform> xf;
    std::vector<int32_t> order;
    std::vector<RagItem> items;
    TwiddleBuilder tb;
    int64_t ws_floats2 = 0;
    int smem = 0;
    int ctas = 0;  // persistent CTAs for `smem` (0: not computed yet)
    int ctas_smem = -1;
    int nlong = 0;
    int64_t in_min = 0, out_min = 0;
    bool autotune = true, use_graph = true, tuned = false;
    long long wait_cycles = 1ll << 31;  // bound of each dependency wait
    int need_bias = 0;                  // test hook: unreachable dependency counts
    cudaStream_t stream = nullptr;
    // device state
    bool dev_ready = false;
    int device = -1;
    void* tw = nullptr;
    RagClass* d_cls = nullptr;
    RagXform* d_xf = nullptr;
    int32_t* d_order = nullptr;
    RagItem* d_items = nullptr;
    int* d_queue = nullptr;
    int* d_err = nullptr;
    float2* d_ws = nullptr;
    cudaStream_t s_cap = nullptr;
    cudaGraphExec_t gexec = nullptr;
    void* g_in = nullptr;
    void* g_out = nullptr;
    int g_inv = -1;
    cudaStream_t g_stream = nullptr;
};

namespace {

void free_device(aclfftRaggedPlan_t* p)
{
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->s_cap) cudaStreamDestroy(p->s_cap);
    for (void* q : {(void*)p->tw, (void*)p->d_cls, (void*)p->d_xf, (void*)p->d_order, (void*)p->d_items,
                    (void*)p->d_queue, (void*)p->d_err, (void*)p->d_ws})
        if (q) cudaFree(q);
    p->gexec = nullptr;
    p->s_cap = nullptr;
    p->tw = nullptr;
    p->d_cls = nullptr;
    p->d_xf = nullptr;
    p->d_order = nullptr;
    p->d_items = nullptr;
    p->d_queue = nullptr;
    p->d_err = nullptr;
    p->d_ws = nullptr;
    p->dev_ready = false;
}

int ctas_for(aclfftRaggedPlan_t* p, int smem);

// The captured graph bakes in the kernel arguments: settings that change
// them force a new capture at the next exec.
void drop_graph(aclfftRaggedPlan_t* p)
{
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    p->gexec = nullptr;
    p->g_in = p->g_out = nullptr;
    p->g_inv = -1;
}

// Shared memory an item of the class needs with the chosen variants: the
// data buffers, then the staged pass-table window.
int class_smem(const RagClass& c)
{
    if (c.mode == RAG_MODE_SINGLE) return (2 * c.group * c.pitch + c.tw_cnt) * 8;
    const int p1 = (2 * c.L1 * (c.group + 1) + c.tw_cnt) * 8;
    const int p2 = (2 * c.group2 * c.pitch + c.tw2_cnt) * 8;
    return std::max(p1, p2);
}

// Contiguous range of the twiddle blob used by an on-chip plan's passes
// (cnt = 0 when it is too wide to stage).
void tw_window(const InnerPlan& ip, int64_t& lo, int32_t& cnt)
{
    int64_t a = -1, b = -1;
    for (int q = 0; q < ip.npass; ++q) {
        const PassDesc& d = ip.pass[q];
        if (d.ns <= 1) continue;
        a = a < 0 ? d.tw_off : std::min<int64_t>(a, d.tw_off);
        b = std::max<int64_t>(b, d.tw_off + (int64_t)d.ns * d.radix);
    }
    lo = a < 0 ? 0 : a;
    cnt = (a < 0 || b - a > kMaxTwWindow) ? 0 : (int32_t)(b - a);
}

// Applies candidate choice ch to the class's device descriptor.
bool apply_choice(ClassPlan& cp, Choice ch)
{
    RagClass& c = cp.dev;
    if (ch.v1 < 0 || ch.v1 >= (int)cp.ip1.size()) return false;
    c.ip = cp.ip1[ch.v1];
    tw_window(c.ip, c.tw_lo, c.tw_cnt);
    c.tw2_lo = 0;
    c.tw2_cnt = 0;
    const int budget = kSmemBudget / 8;  // float2 entries
    if (c.mode == RAG_MODE_SINGLE) {
        c.pitch = row_pitch(c.L);
        int g = std::max(1, kThreads / c.ip.nthr);
        while (g > 1 && 2 * g * c.pitch + c.tw_cnt > budget) --g;
        if (2 * g * c.pitch + c.tw_cnt > budget) c.tw_cnt = 0;
        c.group = g;
        c.group2 = 0;
        c.tw_smem = 2 * g * c.pitch;
    } else {
        if (ch.v2 < 0 || ch.v2 >= (int)cp.ip2.size()) return false;
        c.ip2 = cp.ip2[ch.v2];
        tw_window(c.ip2, c.tw2_lo, c.tw2_cnt);
        int g = std::max(1, kThreads / c.ip.nthr);
        g = std::min(g, c.L2);
        while (g > 1 && 2 * c.L1 * (g + 1) + c.tw_cnt > budget) --g;
        if (2 * c.L1 * (g + 1) + c.tw_cnt > budget) c.tw_cnt = 0;
        c.group = g;
        c.tw_smem = 2 * c.L1 * (g + 1);
        c.pitch = row_pitch(c.L2);
        int g2 = std::max(1, kThreads / c.ip2.nthr);
        g2 = std::min(g2, c.L1);
        while (g2 > 1 && 2 * g2 * c.pitch + c.tw2_cnt > budget) --g2;
        if (2 * g2 * c.pitch + c.tw2_cnt > budget) c.tw2_cnt = 0;
        c.group2 = g2;
        c.tw2_smem = 2 * g2 * c.pitch;
    }
    cp.choice = ch;
    return class_smem(c) <= kSmemBudget;
}

double class_cost(const RagClass& c) { return (double)c.L * std::log2((double)std::max(c.L, 2)); }

void build_items(aclfftRaggedPlan_t* p)
{
    p->items.clear();
    p->order.clear();
    std::vector<RagItem> p1, single, p2, post;
    std::vector<std::pair<double, RagItem>> singles;
    std::vector<int> np1(p->count, 0), np2(p->count, 0);
    for (int ci = 0; ci < (int)p->classes.size(); ++ci) {
        ClassPlan& cp = p->classes[ci];
        const RagClass& c = cp.dev;
        if (c.mode == RAG_MODE_SINGLE) {
            for (size_t i = 0; i < cp.members.size(); i += c.group) {
                RagItem it{};
                it.kind = RAG_SINGLE;
                it.cls = ci;
                it.first = (int)p->order.size();
                it.count = (int)std::min<size_t>(c.group, cp.members.size() - i);
                for (int k = 0; k < it.count; ++k) p->order.push_back(cp.members[i + k]);
                singles.push_back({class_cost(c) * it.count, it});
            }
        } else {
            for (int x : cp.members) {
                for (int j = 0; j < c.L2; j += c.group) {
                    RagItem it{};
                    it.kind = RAG_P1;
                    it.cls = ci;
                    it.first = j;
                    it.count = std::min(c.group, c.L2 - j);
                    it.xform = x;
                    p1.push_back(it);
                    ++np1[x];
                }
                for (int k = 0; k < c.L1; k += c.group2) {
                    RagItem it{};
                    it.kind = RAG_P2;
                    it.cls = ci;
                    it.first = k;
                    it.count = std::min(c.group2, c.L1 - k);
                    it.xform = x;
                    p2.push_back(it);
                    ++np2[x];
                }
                if (c.type == RAG_R2C && !(c.n & 1)) {
                    RagItem it{};
                    it.kind = RAG_POST;
                    it.cls = ci;
                    it.xform = x;
                    post.push_back(it);
                }
            }
        }
    }
    std::stable_sort(singles.begin(), singles.end(),
                     [](const std::pair<double, RagItem>& a, const std::pair<double, RagItem>& b) {
                         return a.first > b.first;
                     });
    for (auto& it : p2) it.need = np1[it.xform];
    for (auto& it : post) it.need = np1[it.xform] + np2[it.xform];
    p->items.insert(p->items.end(), p1.begin(), p1.end());
    for (auto& s : singles) p->items.push_back(s.second);
    p->items.insert(p->items.end(), p2.begin(), p2.end());
    p->items.insert(p->items.end(), post.begin(), post.end());
    p->smem = 16;
    for (auto& cp : p->classes) p->smem = std::max(p->smem, class_smem(cp.dev));
}

template <class T>
bool upload(T*& d, const std::vector<T>& h)
{
    if (d) cudaFree(d);
    d = nullptr;
    const size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
    if (gfft::dev_alloc(reinterpret_cast<void**>(&d), bytes) != cudaSuccess) {
        cudaGetLastError();
        d = nullptr;
        return false;
    }
    if (!h.empty() && cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return true;
}

bool upload_tables(aclfftRaggedPlan_t* p)
{
    std::vector<RagClass> cls;
    for (auto& cp : p->classes) cls.push_back(cp.dev);
    return upload(p->d_cls, cls) && upload(p->d_xf, p->xf) && upload(p->d_order, p->order) &&
           upload(p->d_items, p->items);
}

aclfftResult device_setup(aclfftRaggedPlan_t* p)
{
    if (p->dev_ready) return ACLFFT_SUCCESS;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_SETUP_FAILED;
    }
    const size_t twb = (size_t)std::max<int64_t>(p->tb.count, 2) * 8;
    if (gfft::dev_alloc(&p->tw, twb) != cudaSuccess || gfft::dev_alloc(reinterpret_cast<void**>(&p->d_queue),
                                                             (size_t)(p->count + 1) * sizeof(int)) != cudaSuccess ||
        gfft::dev_alloc(reinterpret_cast<void**>(&p->d_err), sizeof(int)) != cudaSuccess ||
        cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess ||
        (p->ws_floats2 > 0 &&
         gfft::dev_alloc(reinterpret_cast<void**>(&p->d_ws), (size_t)p->ws_floats2 * sizeof(float2)) != cudaSuccess) ||
        cudaStreamCreateWithFlags(&p->s_cap, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        free_device(p);
        gfft::set_last_error("ragged plan: device allocation failed");
        return ACLFFT_ALLOC_FAILED;
    }
    if (!p->tb.segs.empty() && (gfft_gen_twiddles(p->tw, p->tb.segs.data(), (int)p->tb.segs.size(), nullptr) != 0 ||
                                cudaDeviceSynchronize() != cudaSuccess)) {
        cudaGetLastError();
        free_device(p);
        gfft::set_last_error("ragged plan: twiddle generation failed");
        return ACLFFT_SETUP_FAILED;
    }
    if (!upload_tables(p)) {
        free_device(p);
        gfft::set_last_error("ragged plan: table upload failed");
        return ACLFFT_ALLOC_FAILED;
    }
    p->device = dev;
    p->ctas = ctas_for(p, p->smem);
    p->ctas_smem = p->smem;
    if (p->ctas <= 0) {
        free_device(p);
        return ACLFFT_SETUP_FAILED;
    }
    p->dev_ready = true;
    return ACLFFT_SUCCESS;
}

// Persistent CTAs for a shared-memory size (attribute calls: not inside a
// stream capture).
int ctas_for(aclfftRaggedPlan_t* p, int smem)
{
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device < 0 ? 0 : p->device) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    const int per_sm = gfft_ragged_ctas(smem);
    if (per_sm <= 0) {
        gfft::set_last_error(std::string("ragged kernel setup: ") +
                             (per_sm < 0 ? cudaGetErrorString((cudaError_t)(-per_sm)) : "no CTA fits an SM"));
        return 0;
    }
    return per_sm * sms;
}

RagArgs make_args(aclfftRaggedPlan_t* p, const RagItem* items, int nitems, int smem, const void* in, void* out,
                  bool inverse)
{
    RagArgs a{};
    a.cls = p->d_cls;
    a.xf = p->d_xf;
    a.order = p->d_order;
    a.items = items;
    a.nitems = nitems;
    a.smem_bytes = smem;
    a.ctas = smem == p->ctas_smem ? p->ctas : ctas_for(p, smem);
    a.queue = p->d_queue;
    a.err = p->d_err;
    a.tw = p->tw;
    a.in = in;
    a.out = out;
    a.ws = p->d_ws;
    a.inverse = inverse ? 1 : 0;
    a.scale_c2c = 1.f;
    a.wait_cycles = p->wait_cycles;
    a.need_bias = p->need_bias;
    return a;
}

int launch(aclfftRaggedPlan_t* p, const RagArgs& a, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(p->d_queue, 0, (size_t)(p->count + 1) * sizeof(int), st);
    if (e != cudaSuccess) return (int)e;
    return gfft_launch_ragged(&a, st);
}

// Times every candidate of every class on its own trial batch: m copies of
// the class's transform (m * n ~ 2^20 points, so a trial launch runs
// several waves like the real batch does) in scratch buffers, with their
// own queue, transform table and workspace.  The fastest candidate is kept
// and cached by (kind, length).
aclfftResult autotune(aclfftRaggedPlan_t* p)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_tune_file();
    constexpr int64_t kTrialPoints = 1 << 20;
    auto trial_m = [&](const RagClass& c) { return (int)std::min<int64_t>(2048, std::max<int64_t>(4, kTrialPoints / c.n)); };
    auto ws_per = [](const RagClass& c) -> int64_t {
        if (c.mode != RAG_MODE_LONG) return 0;
        return (c.type == RAG_R2C && !(c.n & 1)) ? 2 * (int64_t)c.L : c.L;
    };
    int64_t scratch = 16, wsmax = 1;
    int maxm = 1;
    for (auto& cp : p->classes) {
        const int m = trial_m(cp.dev);
        maxm = std::max(maxm, m);
        scratch = std::max<int64_t>(scratch, (int64_t)m * ((int64_t)cp.dev.n + 2) * 8);
        wsmax = std::max<int64_t>(wsmax, (int64_t)m * ws_per(cp.dev));
    }
    void *sin = nullptr, *sout = nullptr;
    int* squeue = nullptr;
    float2* sws = nullptr;
    RagXform* sxf = nullptr;
    int32_t* sorder = nullptr;
    RagItem* sitems = nullptr;
    RagClass* scls = nullptr;
    size_t cap_xf = 0, cap_order = 0, cap_items = 0, cap_cls = 0;
    bool ok = gfft::dev_alloc(&sin, (size_t)scratch) == cudaSuccess && gfft::dev_alloc(&sout, (size_t)scratch) == cudaSuccess &&
              cudaMemset(sin, 0, (size_t)scratch) == cudaSuccess &&
              gfft::dev_alloc(reinterpret_cast<void**>(&squeue), (size_t)(maxm + 1) * sizeof(int)) == cudaSuccess &&
              gfft::dev_alloc(reinterpret_cast<void**>(&sws), (size_t)wsmax * sizeof(float2)) == cudaSuccess;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ok = ok && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
    for (int ci = 0; ci < (int)p->classes.size() && ok; ++ci) {
        ClassPlan& cp = p->classes[ci];
        const Key key{cp.dev.type, cp.dev.n};
        auto hit = g_tuned.find(key);
        if (hit != g_tuned.end() && apply_choice(cp, hit->second)) {
            cp.tuned = true;
            continue;
        }
        const int n1 = (int)cp.cand1.size();
        const int n2 = cp.dev.mode == RAG_MODE_LONG ? (int)cp.cand2.size() : 1;
        if (n1 * n2 <= 1) continue;
        const int m = trial_m(cp.dev);
        // the trial batch: one class (index 0), m transforms packed in scratch
        aclfftRaggedPlan_t tmp;
        tmp.count = m;
        tmp.xf.resize(m);
        for (int k = 0; k < m; ++k) {
            RagXform& x = tmp.xf[k];
            x.in_off = (int64_t)k * ((int64_t)cp.dev.n + 2) * 8;
            x.out_off = x.in_off;
            x.ws_off = (int64_t)k * ws_per(cp.dev);
            x.cls = 0;
        }
        double best = 1e30;
        Choice bestc = cp.choice;
        for (int a1 = 0; a1 < n1 && ok; ++a1)
            for (int a2 = 0; a2 < n2 && ok; ++a2) {
                if (!apply_choice(cp, {a1, a2})) continue;
                tmp.classes.assign(1, cp);
                tmp.classes[0].members.resize(m);
                for (int k = 0; k < m; ++k) tmp.classes[0].members[k] = k;
                build_items(&tmp);
                std::vector<RagClass> cls(1, cp.dev);
                // trial tables: reallocated only when they grow
                auto put = [&](auto*& d, size_t& cap, const auto& h) {
                    using T = typename std::decay_t<decltype(h)>::value_type;
                    if (h.size() > cap) {
                        if (d) cudaFree(d);
                        d = nullptr;
                        cap = 0;
                        if (gfft::dev_alloc(reinterpret_cast<void**>(&d), h.size() * sizeof(T)) != cudaSuccess) return false;
                        cap = h.size();
                    }
                    return h.empty() ||
                           cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
                };
                if (!put(scls, cap_cls, cls) || !put(sxf, cap_xf, tmp.xf) || !put(sorder, cap_order, tmp.order) ||
                    !put(sitems, cap_items, tmp.items)) {
                    ok = false;
                    break;
                }
                RagArgs ra{};
                ra.cls = scls;
                ra.xf = sxf;
                ra.order = sorder;
                ra.items = sitems;
                ra.nitems = (int)tmp.items.size();
                ra.smem_bytes = tmp.smem;
                ra.ctas = ctas_for(p, tmp.smem);
                ra.queue = squeue;
                ra.err = p->d_err;
                ra.tw = p->tw;
                ra.in = sin;
                ra.out = sout;
                ra.ws = sws;
                ra.scale_c2c = 1.f;
                ra.wait_cycles = 1ll << 31;  // trials never use the plan's test settings
                ra.need_bias = 0;
                if (ra.ctas <= 0) {
                    ok = false;
                    break;
                }
                float tbest = 1e30f;
                for (int rep = 0; rep < 3 && ok; ++rep) {
                    ok = cudaMemsetAsync(squeue, 0, (size_t)(m + 1) * sizeof(int), p->s_cap) == cudaSuccess &&
                         cudaEventRecord(e0, p->s_cap) == cudaSuccess && gfft_launch_ragged(&ra, p->s_cap) == 0 &&
                         cudaEventRecord(e1, p->s_cap) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess;
                    float ms = 0;
                    if (ok) cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) tbest = std::min(tbest, ms);
                }
                if (tbest < best) {
                    best = tbest;
                    bestc = {a1, a2};
                }
            }
        if (!ok) break;
        apply_choice(cp, bestc);
        cp.tuned = true;
        g_tuned[key] = bestc;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    for (void* q : {(void*)sin, (void*)sout, (void*)squeue, (void*)sws, (void*)sxf, (void*)sorder, (void*)sitems,
                    (void*)scls})
        if (q) cudaFree(q);
    if (!ok) {
        cudaGetLastError();
        for (auto& cp : p->classes) {
            apply_choice(cp, {0, 0});
            cp.tuned = false;
        }
    } else {
        save_tune_file();
        p->tuned = true;
    }
    build_items(p);
    if (p->gexec) {
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
    }
    p->ctas = ctas_for(p, p->smem);
    p->ctas_smem = p->smem;
    if (!upload_tables(p)) return ACLFFT_ALLOC_FAILED;
    if (!ok) {
        gfft::set_last_error("ragged autotune: a trial launch failed");
        return ACLFFT_EXEC_FAILED;
    }
    return ACLFFT_SUCCESS;
}

// Device memory of device `dev` (any device when dev < 0) or managed
// memory; another GPU's memory would be dereferenced as a peer address.
bool device_pointer(const void* ptr, int dev)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeManaged) return true;
    return at.type == cudaMemoryTypeDevice && (dev < 0 || at.device == dev);
}

}  // namespace

extern "C" {

ACLFFT_API aclfftResult aclfftRaggedPlanCreate(aclfftRaggedPlan* plan, int count, const int* lengths,
                                               const aclfftType* types, const long long* inOffsets,
                                               const long long* outOffsets)
{
    ACLFFT_CHECK_NULL(plan);
    *plan = nullptr;
    ACLFFT_CHECK_PARAM(count >= 1, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_NULL(lengths);
    ACLFFT_CHECK_NULL(types);
    ACLFFT_CHECK_NULL(inOffsets);
    ACLFFT_CHECK_NULL(outOffsets);
    for (int i = 0; i < count; ++i) {
        ACLFFT_CHECK_PARAM(types[i] == ACLFFT_C2C || types[i] == ACLFFT_R2C, ACLFFT_INVALID_TYPE);
        ACLFFT_CHECK_PARAM(lengths[i] >= 2 && lengths[i] <= kMaxLength, ACLFFT_INVALID_SIZE);
        ACLFFT_CHECK_PARAM(inOffsets[i] >= 0 && outOffsets[i] >= 0, ACLFFT_INVALID_VALUE);
        ACLFFT_CHECK_PARAM(inOffsets[i] % 8 == 0 && outOffsets[i] % 8 == 0, ACLFFT_INVALID_VALUE);
        if (!primes_le_13(lengths[i])) {
            gfft::set_last_error("ragged batches take lengths whose prime factors are <= 13");
            return ACLFFT_NOT_SUPPORTED;
        }
    }
    auto* p = new (std::nothrow) aclfftRaggedPlan_t();
    if (!p) return ACLFFT_ALLOC_FAILED;
    p->count = count;
    p->len.assign(lengths, lengths + count);
    p->in_off.assign(inOffsets, inOffsets + count);
    p->out_off.assign(outOffsets, outOffsets + count);
    p->type.resize(count);
    p->xf.resize(count);
    std::map<Key, int> cidx;
    for (int i = 0; i < count; ++i) {
        const int t = types[i] == ACLFFT_C2C ? RAG_C2C : RAG_R2C;
        p->type[i] = t;
        const int n = lengths[i];
        const Key k{t, n};
        auto f = cidx.find(k);
        int ci;
        if (f == cidx.end()) {
            ci = (int)p->classes.size();
            cidx[k] = ci;
            ClassPlan cp;
            RagClass& c = cp.dev;
            c.n = n;
            c.type = t;
            c.L = (t == RAG_R2C && !(n & 1)) ? n / 2 : n;
            c.post_off = -1;
            c.hi_off = c.lo_off = -1;
            if (c.L <= kMaxSingle) {
                c.mode = RAG_MODE_SINGLE;
                cp.cand1 = candidates(c.L, kThreads);
            } else {
                c.mode = RAG_MODE_LONG;
                // L1 <= L2: the column step (strided) is the shorter one
                int L1 = 1;
                for (int d = 2; (int64_t)d * d <= c.L; ++d)
                    if (c.L % d == 0) L1 = d;
                c.L1 = L1;
                c.L2 = c.L / L1;
                if (c.L2 > kMaxSingle || c.L1 < 2) {
                    delete p;
                    gfft::set_last_error("ragged batches: length does not split into two on-chip factors");
                    return ACLFFT_NOT_SUPPORTED;
                }
                cp.cand1 = candidates(c.L1, kThreads);
                cp.cand2 = candidates(c.L2, kThreads);
                int sh = 0;
                while ((int64_t(1) << (2 * sh)) < c.L) ++sh;
                c.otw_shift = sh;
                c.hi_off = p->tb.add_linear(((c.L - 1) >> sh) + 1, c.L, int64_t(1) << sh);
                c.lo_off = p->tb.add_linear(int64_t(1) << sh, c.L, 1);
            }
            if (t == RAG_R2C && !(n & 1)) c.post_off = p->tb.add_linear(c.L / 2 + 1, n, 1);
            for (auto& v : cp.cand1) {
                InnerPlan ip;
                if (!build_inner(c.mode == RAG_MODE_SINGLE ? c.L : c.L1, v.rad, v.nthr, p->tb, ip)) {
                    delete p;
                    return ACLFFT_INTERNAL_ERROR;
                }
                cp.ip1.push_back(ip);
            }
            for (auto& v : cp.cand2) {
                InnerPlan ip;
                if (!build_inner(c.L2, v.rad, v.nthr, p->tb, ip)) {
                    delete p;
                    return ACLFFT_INTERNAL_ERROR;
                }
                cp.ip2.push_back(ip);
            }
            if (cp.ip1.empty() || (c.mode == RAG_MODE_LONG && cp.ip2.empty()) || !apply_choice(cp, {0, 0})) {
                delete p;
                gfft::set_last_error("ragged batches: no on-chip plan for a length");
                return ACLFFT_NOT_SUPPORTED;
            }
            p->classes.push_back(cp);
        } else {
            ci = f->second;
        }
        p->classes[ci].members.push_back(i);
        RagXform& x = p->xf[i];
        x.in_off = inOffsets[i];
        x.out_off = outOffsets[i];
        x.cls = ci;
        x.ws_off = -1;
        const RagClass& c = p->classes[ci].dev;
        if (c.mode == RAG_MODE_LONG) {
            ++p->nlong;
            x.ws_off = p->ws_floats2;
            p->ws_floats2 += (t == RAG_R2C && !(n & 1)) ? 2 * (int64_t)c.L : c.L;
        }
        const int64_t in_b = t == RAG_C2C ? (int64_t)n * 8 : (int64_t)n * 4;
        const int64_t out_b = t == RAG_C2C ? (int64_t)n * 8 : ((int64_t)n / 2 + 1) * 8;
        p->in_min = std::max(p->in_min, (int64_t)inOffsets[i] + in_b);
        p->out_min = std::max(p->out_min, (int64_t)outOffsets[i] + out_b);
    }
    build_items(p);
    *plan = p;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftRaggedSetStream(aclfftRaggedPlan plan, cudaStream_t stream)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    plan->stream = stream;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftRaggedSetOptions(aclfftRaggedPlan plan, int autotune_on, int use_graph)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    plan->autotune = autotune_on != 0;
    plan->use_graph = use_graph != 0;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftRaggedAutotune(aclfftRaggedPlan plan)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    const aclfftResult r = device_setup(plan);
    if (r != ACLFFT_SUCCESS) return r;
    return autotune(plan);
}

ACLFFT_API aclfftResult aclfftRaggedExec(aclfftRaggedPlan plan, void* idata, void* odata, int direction)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(idata);
    ACLFFT_CHECK_NULL(odata);
    ACLFFT_CHECK_PARAM(direction == ACLFFT_FORWARD || direction == ACLFFT_BACKWARD, ACLFFT_INVALID_VALUE);
    if (!device_pointer(idata, -1) || !device_pointer(odata, -1)) {
        gfft::set_last_error("ragged exec takes device pointers");
        return ACLFFT_INVALID_VALUE;
    }
    aclfftResult r = device_setup(plan);
    if (r != ACLFFT_SUCCESS) return r;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != plan->device) {
        cudaGetLastError();
        return ACLFFT_INVALID_DEVICE;
    }
    if (!device_pointer(idata, dev) || !device_pointer(odata, dev)) {
        gfft::set_last_error("ragged exec takes device pointers of the plan's device");
        return ACLFFT_INVALID_VALUE;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(plan->stream, &cs) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    const bool capturing = cs != cudaStreamCaptureStatusNone;
    if (plan->autotune && !plan->tuned && !capturing) {
        r = autotune(plan);
        if (r != ACLFFT_SUCCESS) return r;
    }
    const bool inv = direction == ACLFFT_BACKWARD;
    const RagArgs a = make_args(plan, plan->d_items, (int)plan->items.size(), plan->smem, idata, odata, inv);
    auto fail = [&](const char* what, int rc) {
        gfft::set_last_error(std::string("ragged exec: ") + what + ": " + cudaGetErrorString((cudaError_t)rc));
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    };
    if (!plan->use_graph || capturing) {
        const int rc = launch(plan, a, plan->stream);
        return rc == 0 ? ACLFFT_SUCCESS : fail("launch", rc);
    }
    if (!plan->gexec || plan->g_in != idata || plan->g_out != odata || plan->g_inv != (int)inv) {
        if (plan->gexec) cudaGraphExecDestroy(plan->gexec);
        plan->gexec = nullptr;
        cudaGraph_t g = nullptr;
        const cudaError_t eb = cudaStreamBeginCapture(plan->s_cap, cudaStreamCaptureModeThreadLocal);
        if (eb != cudaSuccess) return fail("begin capture", (int)eb);
        const int lrc = launch(plan, a, plan->s_cap);
        const cudaError_t ec = cudaStreamEndCapture(plan->s_cap, &g);
        const cudaError_t ei = (lrc == 0 && ec == cudaSuccess) ? cudaGraphInstantiate(&plan->gexec, g, 0) : cudaSuccess;
        if (lrc != 0 || ec != cudaSuccess || ei != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            plan->gexec = nullptr;
            return fail("graph capture", lrc != 0 ? lrc : (ec != cudaSuccess ? (int)ec : (int)ei));
        }
        cudaGraphDestroy(g);
        plan->g_in = idata;
        plan->g_out = odata;
        plan->g_inv = (int)inv;
    }
    const cudaError_t el = cudaGraphLaunch(plan->gexec, plan->stream);
    if (el != cudaSuccess) return fail("graph launch", (int)el);
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftRaggedGetInfo(aclfftRaggedPlan plan, aclfftRaggedInfo* info)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(info);
    std::memset(info, 0, sizeof(*info));
    info->transforms = plan->count;
    info->classes = (int)plan->classes.size();
    info->long_transforms = plan->nlong;
    info->items = (int)plan->items.size();
    for (auto& cp : plan->classes) info->tuned_classes += cp.tuned ? 1 : 0;
    info->workspace_bytes = (size_t)plan->ws_floats2 * 8;
    info->in_bytes_min = (size_t)plan->in_min;
    info->out_bytes_min = (size_t)plan->out_min;
    info->graph = plan->gexec ? 1 : 0;
    info->smem_bytes = plan->smem;
    info->twiddle_entries = plan->tb.count;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftRaggedGetError(aclfftRaggedPlan plan, int* flags)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(flags);
    *flags = 0;
    if (!plan->dev_ready) return ACLFFT_SUCCESS;
    // ordered after the plan's launches: the read is queued on the plan's
    // stream (which may be a non-blocking stream the legacy default stream
    // does not wait for) and that stream is synchronised
    int v = 0;
    if (cudaMemcpyAsync(&v, plan->d_err, sizeof(int), cudaMemcpyDeviceToHost, plan->stream) != cudaSuccess ||
        cudaStreamSynchronize(plan->stream) != cudaSuccess) {
        cudaGetLastError();
        gfft::set_last_error("ragged: reading the device error word failed");
        return ACLFFT_EXEC_FAILED;
    }
    *flags = v;
    if (v == 0) return ACLFFT_SUCCESS;
    if (cudaMemsetAsync(plan->d_err, 0, sizeof(int), plan->stream) != cudaSuccess ||
        cudaStreamSynchronize(plan->stream) != cudaSuccess)
        cudaGetLastError();
    gfft::set_last_error("ragged: a dependency wait ran out of time; the output is incomplete");
    return ACLFFT_EXEC_FAILED;
}

ACLFFT_API aclfftResult aclfftRaggedSetWaitLimit(aclfftRaggedPlan plan, long long cycles)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_PARAM(cycles > 0, ACLFFT_INVALID_VALUE);
    if (plan->wait_cycles != cycles) drop_graph(plan);
    plan->wait_cycles = cycles;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftRaggedDebugHoldDependencies(aclfftRaggedPlan plan, int extra)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_PARAM(extra >= 0, ACLFFT_INVALID_VALUE);
    if (plan->need_bias != extra) drop_graph(plan);
    plan->need_bias = extra;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftRaggedDestroy(aclfftRaggedPlan plan)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    free_device(plan);
    delete plan;
    return ACLFFT_SUCCESS;
}

// Host replay of every item's accesses: input/output extents per transform,
// workspace ranges, table ranges, thread and shared-memory limits, and the
// queue order of dependent items.
ACLFFT_API int aclfftRaggedDebugCheck(aclfftRaggedPlan plan, char* msg, int msglen)
{
    auto report = [&](const std::string& s, int rc) {
        if (msg && msglen > 0) std::snprintf(msg, (size_t)msglen, "%s", s.c_str());
        return rc;
    };
    if (!plan) return report("no plan", -1);
    const int64_t twn = plan->tb.count;
    std::vector<int> seen_p1(plan->count, 0), seen_p2(plan->count, 0);
    for (size_t ii = 0; ii < plan->items.size(); ++ii) {
        const RagItem& it = plan->items[ii];
        if (it.cls < 0 || it.cls >= (int)plan->classes.size()) return report("item class", 1);
        const RagClass& c = plan->classes[it.cls].dev;
        if (class_smem(c) > plan->smem || plan->smem > kSmemBudget) return report("shared memory", 2);
        auto tw_ok = [&](const InnerPlan& ip) {
            for (int q = 0; q < ip.npass; ++q)
                if (ip.pass[q].tw_off >= 0 && ip.pass[q].tw_off + (int64_t)ip.pass[q].ns * ip.pass[q].radix > twn)
                    return false;
            return ip.nthr >= 1 && ip.nthr <= kThreads;
        };
        if (!tw_ok(c.ip)) return report("pass tables / threads", 3);
        if (c.tw_cnt < 0 || c.tw_lo + c.tw_cnt > twn || c.tw2_cnt < 0 || c.tw2_lo + c.tw2_cnt > twn)
            return report("staged twiddle window", 3);
        auto window_covers = [](const InnerPlan& ip, int64_t lo, int cnt) {
            if (cnt == 0) return true;
            for (int q = 0; q < ip.npass; ++q)
                if (ip.pass[q].ns > 1 &&
                    (ip.pass[q].tw_off < lo || ip.pass[q].tw_off + (int64_t)ip.pass[q].ns * ip.pass[q].radix > lo + cnt))
                    return false;
            return true;
        };
        if (!window_covers(c.ip, c.tw_lo, c.tw_cnt) ||
            (c.mode == RAG_MODE_LONG && !window_covers(c.ip2, c.tw2_lo, c.tw2_cnt)))
            return report("staged window misses a pass table", 3);
        if (c.post_off >= 0 && c.post_off + c.L / 2 + 1 > twn) return report("post table", 3);
        if (it.kind == RAG_SINGLE) {
            if (c.group * c.ip.nthr > kThreads || it.count < 1 || it.count > c.group) return report("single group", 4);
            if (c.pitch < spad_h(c.L - 1) + 1) return report("pitch", 4);
            if (it.first < 0 || it.first + it.count > (int)plan->order.size()) return report("order range", 4);
            for (int k = 0; k < it.count; ++k) {
                const int x = plan->order[it.first + k];
                if (x < 0 || x >= plan->count || plan->xf[x].cls != it.cls) return report("order entry", 4);
            }
        } else {
            if (it.xform < 0 || it.xform >= plan->count || plan->xf[it.xform].cls != it.cls) return report("xform", 5);
            const RagXform& x = plan->xf[it.xform];
            const int64_t wsn = (c.type == RAG_R2C && !(c.n & 1)) ? 2 * (int64_t)c.L : c.L;
            if (x.ws_off < 0 || x.ws_off + wsn > plan->ws_floats2) return report("workspace", 5);
            if (c.hi_off < 0 || c.hi_off + ((c.L - 1) >> c.otw_shift) + 1 > twn || c.lo_off + (1 << c.otw_shift) > twn)
                return report("outer twiddles", 5);
            if ((int64_t)(c.L1 - 1) * (c.L2 - 1) >= c.L) return report("outer index", 5);
            if (it.kind == RAG_P1) {
                if (c.group * c.ip.nthr > kThreads || it.first + it.count > c.L2) return report("p1 range", 6);
                ++seen_p1[it.xform];
            } else if (it.kind == RAG_P2) {
                if (!tw_ok(c.ip2) || c.group2 * c.ip2.nthr > kThreads || it.first + it.count > c.L1)
                    return report("p2 range", 7);
                if (seen_p1[it.xform] != it.need) return report("p2 queued before its p1 items", 7);
                ++seen_p2[it.xform];
            } else {
                if (seen_p1[it.xform] + seen_p2[it.xform] != it.need) return report("post queued early", 8);
            }
        }
    }
    return report("ok", 0);
}

}  // extern "C"
