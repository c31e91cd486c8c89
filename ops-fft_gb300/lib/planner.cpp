// planner.cpp - see planner.h.
#include "planner.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <functional>

namespace gfft {

namespace {

constexpr int kBigPrimes[] = {17, 19, 23, 29, 31, 37, 41, 43, 47};

int max_threads_for(int rmax) { return rmax <= 16 ? 512 : 256; }

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace

std::vector<int64_t> prime_factors(int64_t n)
{
    std::vector<int64_t> f;
    if (n <= 1) return f;
    for (int64_t p = 2; p * p <= n; ++p) {
        while (n % p == 0) {
            f.push_back(p);
            n /= p;
        }
    }
    if (n > 1) f.push_back(n);
    return f;
}

bool all_primes_at_most(int64_t n, int64_t pmax)
{
    for (int64_t p : prime_factors(n))
        if (p > pmax) return false;
    return true;
}

bool length_supported(int64_t n) { return n >= 1 && all_primes_at_most(n, 47); }

std::vector<int> choose_radices(int L)
{
    if (L == 1) return {1};
    if (!all_primes_at_most(L, 47)) return {};
    std::vector<int> allowed;
    for (int r = 16; r >= 2; --r) allowed.push_back(r);
    for (int p : kBigPrimes)
        if (L % p == 0) allowed.insert(allowed.begin(), p);
    std::sort(allowed.begin(), allowed.end(), std::greater<int>());

    std::vector<int> best, cur;
    int best_pass = 1 << 30, best_min = 0, best_pow2 = -1;
    std::function<void(int, int)> dfs = [&](int rem, int maxr) {
        if ((int)cur.size() > best_pass || (int)cur.size() >= kMaxPass) return;
        if (rem == 1) {
            const int np = (int)cur.size();
            const int mn = *std::min_element(cur.begin(), cur.end());
            int pow2 = 0;
            for (int r : cur) pow2 += ((r & (r - 1)) == 0);
            if (np < best_pass || (np == best_pass && (mn > best_min || (mn == best_min && pow2 > best_pow2)))) {
                best = cur;
                best_pass = np;
                best_min = mn;
                best_pow2 = pow2;
            }
            return;
        }
        for (int r : allowed) {
            if (r > maxr || rem % r) continue;
            cur.push_back(r);
            dfs(rem / r, r);
            cur.pop_back();
        }
    };
    dfs(L, 1 << 30);
    return best;
}

int64_t TwiddleBuilder::add_pass_table(int64_t ns, int R)
{
    // layout [r][k]: entry r*ns + k = W_{ns*R}^{k*r}; consecutive butterflies
    // (consecutive k) read consecutive entries
    for (const TwSeg& t : segs)
        if (t.kind == 2 && t.M == ns * R && t.R_or_mult == ns) return t.offset;
    const int64_t off = count;
    TwSeg s{};
    s.offset = off;
    s.count = ns * R;
    s.M = ns * R;
    s.R_or_mult = ns;
    s.kind = 2;
    segs.push_back(s);
    count += ns * R;
    count += count & 1;
    return off;
}

int64_t TwiddleBuilder::add_linear(int64_t n, int64_t M, int64_t mult)
{
    for (const TwSeg& t : segs)
        if (t.kind == 1 && t.M == M && t.R_or_mult == mult && t.count >= n) return t.offset;
    const int64_t off = count;
    TwSeg s{};
    s.offset = off;
    s.count = n;
    s.M = M;
    s.R_or_mult = mult;
    s.kind = 1;
    segs.push_back(s);
    count += n;
    count += count & 1;
    return off;
}

int64_t TwiddleBuilder::add_dft_matrix(int R, int prec)
{
    for (const TwSeg& t : segs)
        if (t.kind == 3 && t.M == R && t.R_or_mult == prec) return t.offset;
    const int64_t n = gfft_tc_bmat_entries(R, prec);
    if (n <= 0) return -1;
    const int64_t off = count;
    TwSeg s{};
    s.offset = off;
    s.count = n;
    s.M = R;
    s.R_or_mult = prec;
    s.kind = 3;
    segs.push_back(s);
    count += n;
    count += count & 1;
    return off;
}

int64_t TwiddleBuilder::add_dtable(int64_t n)
{
    for (const auto& d : dsegs)
        if (d.second == n) return d.first;
    const int64_t off = count;
    dsegs.emplace_back(off, n);
    count += 2 * n;
    return off;
}

bool build_inner(int L, const std::vector<int>& radices, int nthr, TwiddleBuilder& tb, InnerPlan& ip)
{
    if (radices.empty() || (int)radices.size() > kMaxPass) return false;
    ip = InnerPlan{};
    ip.L = L;
    ip.npass = (int)radices.size();
    ip.nthr = nthr;
    ip.rmax = 16;
    int64_t ns = 1;
    for (int p = 0; p < ip.npass; ++p) {
        const int R = radices[p];
        if (R > 16) ip.rmax = 47;
        PassDesc& d = ip.pass[p];
        d.radix = R;
        d.ns = (int32_t)ns;
        d.ns_magic = ns > 1 ? (uint32_t)(((1ull << 32) + (uint64_t)ns - 1) / (uint64_t)ns) : 0u;
        d.tw_off = ns > 1 ? (int32_t)tb.add_pass_table(ns, R) : -1;
        ns *= R;
    }
    return ns == L;
}

namespace {

int pick_nthr(int L, const std::vector<int>& radices, int maxthr)
{
    int nbf_max = 1;
    for (int r : radices) nbf_max = std::max(nbf_max, L / r);
    if (nbf_max <= maxthr) return nbf_max;
    return (int)ceil_div(nbf_max, ceil_div(nbf_max, maxthr));
}

// Shared-memory buffers a row transform needs (see row_body in stockham.cuh).
int row_nbuf(int npass, int start, bool last_global)
{
    const int writes = npass - (last_global ? 1 : 0);
    if (start == 1) return writes >= 1 ? 2 : 1;
    return writes >= 2 ? 2 : 1;
}

}  // namespace

// Hints of the problem being planned (set by build_steps for its duration).
thread_local const PlanHints* t_hints = nullptr;

struct HintScope {
    explicit HintScope(const PlanHints* h) : prev(t_hints) { t_hints = h; }
    ~HintScope() { t_hints = prev; }
    const PlanHints* prev;
};

// Largest lengths accepted by the generic kernels (checked exactly below).
int row_max_length() { return 13312; }

bool codelets_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("OPS_FFT_CODELETS");
        return !(v && v[0] == '0');
    }();
    if (t_hints && t_hints->codelets == 0) return false;
    return on;
}
int col_max_length() { return 2048; }

bool clusters_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("OPS_FFT_CLUSTER");
        return !(v && v[0] == '0');
    }();
    if (t_hints && t_hints->cluster == 0) return false;
    return on;
}

namespace {

// Score bonus of a codelet configuration with a per-group work buffer
// (ping-pong passes) over the in-place one.
constexpr double kPingPongScore = 0.0;

// Codelet row step (see csrc/codelet.cuh for the execution model and the
// shared-memory layout).  Returns false when no codelet applies.
bool make_codelet_step(int L, int64_t ntf, int64_t in_dist, int64_t out_dist, int io_mode, int nreal, int weight,
                       TwiddleBuilder& tb, Step& st)
{
    if (!codelets_enabled()) return false;
    // OPS_FFT_CODELET_VARIANT=k selects the k-th entry of this length
    // (tuning experiments); unset or absent, the first one
    const char* env_var = std::getenv("OPS_FFT_CODELET_VARIANT");
    int want = env_var ? std::atoi(env_var) : 0;
    if (t_hints && t_hints->codelet_variant >= 0) want = t_hints->codelet_variant;
    int id = gfft_codelet_find(L, want);
    if (id < 0) id = gfft_codelet_find(L, 0);
    if (id < 0) return false;
    int cl = 0, cn = 0, cr[kMaxPass], cnr = 0, cmaxt = 0, cminb = 0;
    if (gfft_codelet_info(id, &cl, &cn, cr, &cnr, &cmaxt, &cminb) != 0 || cl != L) return false;
    const std::vector<int> rad(cr, cr + cnr);
    const bool even_mode = io_mode == IO_R2C_EVEN || io_mode == IO_C2R_EVEN;
    const bool staged = false;
    const int pshift = (rad[0] % 2 == 0) ? 4 : 30;
    const int maxidx = even_mode ? L : L - 1;
    int lpad = maxidx + (maxidx >> pshift) + 2;
    lpad += lpad & 1;
    const int esize = io_mode == IO_R2C_ODD ? 4 : 8;
    const int64_t row_bytes = in_dist * esize;
    TwiddleBuilder trial = tb;  // do not register tables unless the codelet is used
    st = Step{};
    st.kind = Step::ROW;
    RowArgs& a = st.row;
    if (!build_inner(L, rad, cn, trial, a.ip)) return false;
    int64_t lo = -1, hi = -1;
    for (int p = 0; p < a.ip.npass; ++p) {
        const PassDesc& d = a.ip.pass[p];
        if (d.ns <= 1) continue;
        lo = lo < 0 ? d.tw_off : std::min<int64_t>(lo, d.tw_off);
        hi = std::max<int64_t>(hi, d.tw_off + (int64_t)d.ns * d.radix);
    }
    const int64_t tw_cnt = lo < 0 ? 0 : hi - lo;
    const int64_t post_cnt = even_mode ? L / 2 + 1 : 0;
    int64_t post_off = -1;
    if (even_mode) post_off = trial.add_linear(L / 2 + 1, 2 * (int64_t)L, 1);
    auto align = [](int64_t x, int64_t a) { return (x + a - 1) / a * a; };
    const int64_t hdr = 128;
    // the tables arrive by bulk copies of their 16-byte aligned supersets
    // (a table starting 8 bytes into a 16-byte unit sits 8 bytes in): one
    // spare 16-byte unit each
    const int64_t tw_bytes = tw_cnt > 0 ? align(tw_cnt * 8 + 16, 16) : 0;
    const int64_t post_bytes = post_cnt > 0 ? align(post_cnt * 8 + 16, 16) : 0;
    const int tps = 1;
    // one transform per slot: raw row at offset src % 16 (< 16), padded work
    // layout from offset 16, both inside the slot
    const int64_t stage_bytes = align(std::max<int64_t>(row_bytes + 32, 16 + (int64_t)lpad * 8), 128);
    const int64_t cta_fixed = align(hdr + tw_bytes + post_bytes, 128);
    const int64_t nslots = (ntf + tps - 1) / tps;
    double best = -1e300;  // any configuration that fits beats none
    int best_ng = 0, best_ns = 0;
    int64_t best_gb = 0;
    // OPS_FFT_CODELET_NG / OPS_FFT_CODELET_NST pin the groups per CTA and
    // prefetch stages (tuning experiments); unset, the score below decides
    const char* env_ng = std::getenv("OPS_FFT_CODELET_NG");
    const char* env_ns = std::getenv("OPS_FFT_CODELET_NST");
    const int force_ng = (t_hints && t_hints->codelet_ng > 0) ? t_hints->codelet_ng : (env_ng ? std::atoi(env_ng) : 0);
    const int force_ns = (t_hints && t_hints->codelet_nst > 0) ? t_hints->codelet_nst : (env_ns ? std::atoi(env_ns) : 0);
    // a per-group work buffer (ping-pong passes, half the group barriers):
    // OPS_FFT_CODELET_PP=0/1 or the autotuner pin it; unset, the score decides
    const char* env_pp = std::getenv("OPS_FFT_CODELET_PP");
    const int force_pp = (t_hints && t_hints->codelet_pp >= 0) ? t_hints->codelet_pp : (env_pp ? std::atoi(env_pp) : -1);
    const int64_t work_bytes = align((int64_t)lpad * 8, 128);
    int best_pp = 0;
    for (int pp = 0; pp <= 1; ++pp)
    for (int nst = 2; nst <= 4; ++nst) {
        if (force_pp >= 0 && pp != force_pp) continue;
        if (force_ns ? nst != force_ns : nst > 3) continue;
        const int64_t gb = align(64 + nst * stage_bytes + (pp ? work_bytes : 0), 128);
        for (int ng = 1; ng <= 15 && ng * cn <= cmaxt; ++ng) {
            if (force_ng && ng != force_ng) continue;
            const int64_t smem = cta_fixed + ng * gb;
            if (smem > kMaxSmemBytes) break;
            const int64_t warps = (int64_t)ng * cn / 32;
            // registers: the launch bound caps each thread at 65536 / (MAXT * MINB);
            // they are allocated per warp in each of the 4 SM sub-partitions
            // (16384 registers each), so resident warps come in multiples of 4
            const int64_t reg_cap = std::min<int64_t>(255, (65536 / ((int64_t)cmaxt * cminb)) & ~(int64_t)7);
            const int64_t warps_by_regs = 4 * (16384 / (reg_cap * 32));
            const int64_t ctas = std::min<int64_t>(
                {(228 * 1024) / (smem + 1024), 64 / warps, 32, warps_by_regs / warps});
            if (ctas < 1) continue;
            int64_t groups_sm = ctas * ng;
            // a small batch cannot keep every group busy
            groups_sm = std::min<int64_t>(groups_sm, std::max<int64_t>(1, (nslots + 151) / 152));
            const double occ = (double)std::min<int64_t>(groups_sm * cn, 1536) / 1536.0;
            // bytes of input copies in flight per SM, saturating at 40 KB
            // (more stages beyond that measured slower: R2C, C2R and the
            // weighted R2C adjoint at N=3000, batch 4096, 4 groups per SM,
            // 2 stages 1-3 % faster than 3)
            const double infl =
                (double)std::min<int64_t>(groups_sm * (nst - 1) * tps * row_bytes, 40 * 1024) / (40 * 1024.0);
            const double score = occ + infl - 0.02 * nst + kPingPongScore * pp;
            // ties: more groups per CTA (up to 384 threads) share the CTA's
            // twiddle tables and hide each other's barriers (measured faster)
            const bool tie_better = score > best - 1e-9 && ng > best_ng && ng * cn <= 384;
            if (score > best + 1e-9 || tie_better) {
                best = score;
                best_ng = ng;
                best_ns = nst;
                best_gb = gb;
                best_pp = pp;
            }
        }
    }
    if (best_ng == 0) return false;
    tb = trial;
    st.post_off = post_off;
    a.ntf = ntf;
    a.in_dist = in_dist;
    a.out_dist = out_dist;
    a.tfpc = tps;
    a.lpad = lpad;
    a.nbuf = best_pp ? 2 : 1;
    a.io_mode = io_mode;
    a.weight = weight;
    a.nreal = nreal;
    a.staged = staged ? 1 : 0;
    a.scale = 1.f;
    a.conj_out = io_mode == IO_C2R_EVEN ? 1 : 0;
    a.nstage = best_ns;
    a.pshift = pshift;
    a.in_esize = esize;
    a.tw_lo = (int32_t)(lo < 0 ? 0 : lo);
    a.tw_cnt = (int32_t)tw_cnt;
    a.post_cnt = (int32_t)post_cnt;
    a.stage_bytes = (int32_t)stage_bytes;
    a.smem_tw = (int32_t)hdr;
    a.smem_post = (int32_t)(hdr + tw_bytes);
    a.smem_stage = (int32_t)cta_fixed;
    a.smem_work = best_pp ? (int32_t)(64 + best_ns * stage_bytes) : 0;  // group offset of the work buffer
    a.group_bytes = (int32_t)best_gb;
    a.ngroups = best_ng;
    a.smem_bytes = (int32_t)(cta_fixed + best_ng * best_gb);
    a.codelet = id;
    st.tw_off = 0;
    return true;
}

// One on-chip transform per contiguous batch item (persistent row kernel,
// see csrc/row_pipe.cuh for the shared-memory layout).
bool make_row_step(int L, int64_t ntf, int64_t in_dist, int64_t out_dist, int io_mode, int nreal, int weight,
                   TwiddleBuilder& tb, Step& st)
{
    std::vector<int> rad = choose_radices(L);
    if (rad.empty()) return false;
    int rmax = *std::max_element(rad.begin(), rad.end()) > 16 ? 47 : 16;
    int maxthr = max_threads_for(rmax);
    int nthr = pick_nthr(L, rad, maxthr);
    int codelet = -1;
    if (make_codelet_step(L, ntf, in_dist, out_dist, io_mode, nreal, weight, tb, st)) return true;
    const bool even_mode = io_mode == IO_R2C_EVEN || io_mode == IO_C2R_EVEN;
    const bool staged = nthr < 32 && (io_mode == IO_C2C || io_mode == IO_R2C_EVEN);
    const int start = io_mode == IO_C2R_EVEN ? 1 : 0;
    const bool last_global = !(io_mode == IO_R2C_EVEN || (io_mode == IO_C2C && staged));
    const int nbuf = std::max(1, row_nbuf((int)rad.size(), start, last_global));
    const int pshift = (rad[0] % 2 == 0) ? 4 : 30;
    const int maxidx = even_mode ? L : L - 1;
    int lpad = maxidx + (maxidx >> pshift) + 2;
    lpad += lpad & 1;
    const int esize = io_mode == IO_R2C_ODD ? 4 : 8;
    const int64_t row_bytes = in_dist * esize;

    st = Step{};
    st.kind = Step::ROW;
    RowArgs& a = st.row;
    if (!build_inner(L, rad, nthr, tb, a.ip)) return false;
    // pass-table window (contiguous range of the blob used by this transform)
    int64_t lo = -1, hi = -1;
    for (int p = 0; p < a.ip.npass; ++p) {
        const PassDesc& d = a.ip.pass[p];
        if (d.ns <= 1) continue;
        const int64_t b0 = d.tw_off, b1 = d.tw_off + (int64_t)d.ns * d.radix;
        lo = lo < 0 ? b0 : std::min(lo, b0);
        hi = std::max(hi, b1);
    }
    const int64_t tw_cnt = lo < 0 ? 0 : hi - lo;
    const bool tw_in_smem = tw_cnt * 8 <= 72 * 1024;

    const int64_t post_cnt = even_mode ? L / 2 + 1 : 0;
    if (even_mode) st.post_off = tb.add_linear(L / 2 + 1, 2 * (int64_t)L, 1);

    auto align = [](int64_t x, int64_t a) { return (x + a - 1) / a * a; };
    const int64_t hdr = 128;
    const int64_t tw_bytes = tw_in_smem ? align(tw_cnt * 8, 16) : 0;
    const int64_t post_bytes = align(post_cnt * 8, 16);
    // tiles must keep the bulk copies 16-byte aligned when rows are not
    int tf_mult = 1;
    while ((row_bytes * tf_mult) % 16 != 0 && tf_mult < 16) tf_mult *= 2;
    const int64_t tmax = std::max<int64_t>(
        1, std::min<int64_t>({(int64_t)maxthr / nthr, std::max<int64_t>(1, (48 * 1024) / row_bytes), ntf}));
    // keep at least ~one tile per SM for small batches
    const int64_t tcap = std::max<int64_t>(1, (ntf + 151) / 152);
    double best = -1;
    int best_tf = 1, best_ns = 1;
    int64_t best_smem = 0;
    for (int ns_ = 1; ns_ <= 3; ++ns_) {
        for (int64_t tf = std::min(tmax, std::max<int64_t>(tcap, 1)); tf >= 1; --tf) {
            const int64_t stage = align(tf * row_bytes, 128);
            const int64_t work = tf * nbuf * (int64_t)lpad * 8;
            const int64_t smem = hdr + tw_bytes + post_bytes + ns_ * stage + work;
            if (smem > kMaxSmemBytes) continue;
            const int64_t threads = tf * nthr;
            const int64_t warps = (threads + 31) / 32;
            const int64_t ctas = std::min<int64_t>({(228 * 1024) / (smem + 1024), 64 / std::max<int64_t>(warps, 1), 32});
            if (ctas < 1) continue;
            const double thr_sm = (double)std::min<int64_t>(ctas * threads, 1024) / 1024.0;
            const double infl = (double)std::min<int64_t>(ctas * (ns_ - 1) * tf * row_bytes, 96 * 1024) / (96 * 1024.0);
            double score = thr_sm + infl + (tf % tf_mult == 0 ? 0.5 : 0.0) + 0.01 * ns_;
            if (score > best) {
                best = score;
                best_tf = (int)tf;
                best_ns = ns_;
                best_smem = smem;
            }
        }
    }
    if (best < 0) return false;
    a.ntf = ntf;
    a.in_dist = in_dist;
    a.out_dist = out_dist;
    a.tfpc = best_tf;
    a.lpad = lpad;
    a.nbuf = nbuf;
    a.io_mode = io_mode;
    a.weight = weight;
    a.nreal = nreal;
    a.staged = staged ? 1 : 0;
    a.scale = 1.f;
    a.conj_out = io_mode == IO_C2R_EVEN ? 1 : 0;
    a.nstage = best_ns;
    a.pshift = pshift;
    a.in_esize = esize;
    a.tw_lo = (int32_t)(lo < 0 ? 0 : lo);
    a.tw_cnt = tw_in_smem ? (int32_t)tw_cnt : 0;
    a.post_cnt = (int32_t)post_cnt;
    a.stage_bytes = (int32_t)align(best_tf * row_bytes, 128);
    a.smem_tw = (int32_t)hdr;
    a.smem_post = (int32_t)(hdr + tw_bytes);
    a.smem_stage = (int32_t)align(hdr + tw_bytes + post_bytes, 128);
    a.smem_work = (int32_t)(a.smem_stage + (int64_t)best_ns * a.stage_bytes);
    a.smem_bytes = (int32_t)(a.smem_work + (int64_t)best_tf * nbuf * lpad * 8);
    a.codelet = codelet;
    a.ngroups = 0;
    a.group_bytes = 0;
    (void)best_smem;
    st.tw_off = 0;
    return a.smem_bytes <= kMaxSmemBytes;
}

// One column pass over an axis of length n (stride S between samples, S
// independent columns per item, `items` items `D` apart).  The pass runs the
// q-th factor Lq of the axis decomposition after a product Ns of earlier
// factors (outer Stockham pass); Ns == 1 and Lq == n is a plain strided
// transform.
bool make_col_step(int64_t n, int64_t S, int64_t items, int64_t D, int Lq, int64_t Ns, TwiddleBuilder& tb, Step& st)
{
    std::vector<int> rad = choose_radices(Lq);
    if (rad.empty()) return false;
    const int rmax = *std::max_element(rad.begin(), rad.end()) > 16 ? 47 : 16;
    const int maxthr = max_threads_for(rmax);
    const bool staged_out = (S == 1 && Ns == 1 && Lq != n);
    const int writes = (int)rad.size() - (staged_out ? 0 : 1);
    const int nbuf = writes >= 2 ? 2 : 1;
    const int64_t cpi = (n / Lq) * S;
    // widest column group that fits
    int tf = 16;
    int nthr = 1;
    for (; tf >= 1; tf >>= 1) {
        const int tfp = tf + 1;
        if ((int64_t)nbuf * Lq * tfp * 8 > kMaxSmemBytes) continue;
        nthr = pick_nthr(Lq, rad, std::max(1, maxthr / tf));
        if (nthr * tf > maxthr) continue;
        if ((int64_t)nbuf * Lq * tfp * 8 > 110 * 1024 && tf > 4) continue;
        break;
    }
    if (tf < 1) return false;
    st = Step{};
    st.kind = Step::COL;
    ColArgs& a = st.col;
    if (!build_inner(Lq, rad, nthr, tb, a.ip)) return false;
    a.ncols = items * cpi;
    a.cpi = cpi;
    a.in_dist = D;
    a.in_split = cpi;
    a.in_hi = 0;
    a.in_lo = 1;
    a.in_stride = (n / Lq) * S;
    a.out_dist = D;
    a.out_split = Ns * S;
    a.out_hi = Ns * Lq * S;
    a.out_lo = 1;
    a.out_stride = Ns * S;
    a.ons = Ns;
    a.tw_div = S;
    a.tfpc = tf;
    a.tfp = tf + 1;
    a.nbuf = nbuf;
    a.staged_out = staged_out ? 1 : 0;
    a.scale = 1.f;
    st.tw_off = 0;
    a.codelet = -1;
    // plain column passes of a length with a codelet run as column tiles of
    // that codelet (one transform group per column, in-place passes)
    if (Ns == 1 && !staged_out && codelets_enabled()) {
        // the codelet of this length whose launch bound holds 8 to 16
        // columns with the most threads resident per SM (independent CTAs
        // overlap one tile's loads with another's passes: 8 columns of 512
        // points at 3 CTAs per SM ran the strided axes of a 512^3 C2C 10 %
        // faster than 16 columns at one), then the most columns (wider
        // tiles read longer row segments); the first such entry on ties
        // (OPS_FFT_COLTILE_VARIANT=k: the k-th codelet of the length, tiles
        // of at least 4 columns; tuning experiments)
        int id = -1, cl = 0, cn = 0, cr[kMaxPass], cnr = 0, cmaxt = 0, cminb = 0;
        const char* env_cv = std::getenv("OPS_FFT_COLTILE_VARIANT");
        int min_tf = 8;
        if (env_cv) {
            const int cand = gfft_codelet_find(Lq, std::atoi(env_cv));
            if (cand >= 0 && gfft_codelet_info(cand, &cl, &cn, cr, &cnr, &cmaxt, &cminb) == 0 && 4 * cn <= cmaxt) {
                id = cand;
                min_tf = 4;
            }
        }
        if (id < 0) {
            int best_cols = 0, best_res = 0;
            for (int k = 0;; ++k) {
                const int cand = gfft_codelet_find(Lq, k);
                if (cand < 0) break;
                if (gfft_codelet_info(cand, &cl, &cn, cr, &cnr, &cmaxt, &cminb) != 0) continue;
                const int cols = std::min(16, cmaxt / cn);
                const int res = cmaxt * cminb;
                if (cols >= 8 && (res > best_res || (res == best_res && cols > best_cols))) {
                    best_cols = cols;
                    best_res = res;
                    id = cand;
                }
            }
            if (id >= 0) gfft_codelet_info(id, &cl, &cn, cr, &cnr, &cmaxt, &cminb);
        }
        if (id >= 0) {
            TwiddleBuilder trial = tb;
            InnerPlan ip;
            const std::vector<int> crad(cr, cr + cnr);
            if (build_inner(Lq, crad, cn, trial, ip)) {
                int64_t lo = -1, hi = -1;
                for (int p = 0; p < ip.npass; ++p) {
                    const PassDesc& d = ip.pass[p];
                    if (d.ns <= 1) continue;
                    lo = lo < 0 ? d.tw_off : std::min<int64_t>(lo, d.tw_off);
                    hi = std::max<int64_t>(hi, d.tw_off + (int64_t)d.ns * d.radix);
                }
                const int64_t tw_cnt = lo < 0 ? 0 : hi - lo;
                const int pshift = (cr[0] % 2 == 0) ? 4 : 30;
                const int64_t wsize = ((int64_t)(Lq - 1) + ((int64_t)(Lq - 1) >> pshift) + 1) | 1;
                int tfc = 1;
                while (tfc * 2 * cn <= cmaxt && tfc < 16) tfc *= 2;
                const int64_t twb = (tw_cnt * 8 + 127) & ~int64_t(127);
                // up to 72 KB per CTA (several CTAs per SM) when the launch bound
                // allows more than one CTA per SM; a single-CTA bound takes all
                const int64_t cap = cminb > 1 ? 72 * 1024 : kMaxSmemBytes;
                while (tfc > 1 && twb + (int64_t)tfc * wsize * 8 > cap) tfc /= 2;
                const int64_t smem = twb + (int64_t)tfc * wsize * 8;
                // tiles narrower than 8 columns (64-byte row segments) lose more to
                // sector granularity than the in-place passes gain (measured on
                // 2048-point columns: 2 columns per tile were 1.7x slower than the
                // column kernel's 4)
                if (tfc >= min_tf && smem <= kMaxSmemBytes && tw_cnt * 8 <= 64 * 1024) {
                    tb = trial;
                    a.ip = ip;
                    a.codelet = id;
                    a.tfpc = tfc;
                    a.tfp = tfc;
                    a.nbuf = 1;
                    a.tw_lo = (int32_t)(lo < 0 ? 0 : lo);
                    a.tw_cnt = (int32_t)tw_cnt;
                    a.wsize = (int32_t)wsize;
                    a.smem_bytes = (int32_t)smem;
                }
            }
        }
    }
    if (Ns > 1) {
        const int64_t M = Ns * Lq;
        int shift = 0;
        while ((int64_t(1) << (2 * shift)) < M) ++shift;  // 2^shift >= sqrt(M)
        a.otw_shift = shift;
        st.lo_off = tb.add_linear(int64_t(1) << shift, M, 1);
        st.hi_off = tb.add_linear(ceil_div(M, int64_t(1) << shift), M, int64_t(1) << shift);
    }
    return true;
}

// Whole batched transform on thread-block clusters (one cluster per
// transform, see csrc/cluster_fft.cuh): a C2C of length n (io_mode IO_C2C)
// or an even R2C / C2R of real length 2n with the packing fused
// (IO_R2C_EVEN / IO_C2R_EVEN).  False when no configuration exists.
bool make_cluster_step(int64_t n, int64_t batch, TwiddleBuilder& tb, Step& st, int io_mode = IO_C2C,
                       int weight = WEIGHT_NONE)
{
    if (!clusters_enabled() || n > 0x7fffffff) return false;
    const char* env_c = std::getenv("OPS_FFT_CLUSTER_C");
    const int want_c = (t_hints && t_hints->cluster_c > 0) ? t_hints->cluster_c : (env_c ? std::atoi(env_c) : 0);
    int C = 0, Q = 0, P = 0, Q0 = 0, P0 = 0, nt = 0, smem = 0;
    const int kid = gfft_cluster_lookup(n, want_c, &C, &Q, &P, &Q0, &P0, &nt, &smem);
    if (kid < 0) return false;
    st = Step{};
    st.kind = Step::CLUSTER;
    ClusterArgs& a = st.cl;
    a.kid = kid;
    a.csize = C;
    a.ntf = batch;
    a.in_dist = io_mode == IO_C2R_EVEN ? n + 1 : n;
    a.out_dist = io_mode == IO_R2C_EVEN ? n + 1 : n;
    a.io_mode = io_mode;
    a.weight = weight;
    a.conj_out = io_mode == IO_C2R_EVEN ? 1 : 0;
    a.post_off = io_mode == IO_C2C ? 0 : tb.add_linear(n + 1, 2 * n, 1);
    a.twq_off = tb.add_pass_table(Q0, Q / Q0);
    a.twp_off = tb.add_pass_table(P0, P / P0);
    a.outer_off = tb.add_linear(n, n, 1);
    a.scale = 1.f;
    a.smem_bytes = smem;
    a.clusters = 0;
    a.length = (int32_t)n;
    st.tw_off = 0;
    return true;
}

// Lengths that a row kernel holds in one thread group (n <= 4096) run on a
// cluster only for batches of at most OPS_FFT_CLUSTER_MAXBATCH transforms
// (default 0: never) or when the autotuner chose it; longer lengths always
// prefer a cluster.  Measured C2C 4096 (us, cluster vs row codelet): b = 8
// 3.57 / 3.62, 64 4.50 / 3.70, 256 7.04 / 5.22, 1024 18.5 / 16.1; R2C 8192
// b = 64 5.44 / 4.17, 256 9.16 / 7.02.
bool cluster_for_batch(int64_t n, int64_t batch)
{
    if (n > 4096) return true;
    if (t_hints && t_hints->cluster == 1) return true;
    const char* v = std::getenv("OPS_FFT_CLUSTER_MAXBATCH");
    return batch <= (v ? (int64_t)std::atoll(v) : (int64_t)0);
}

// Strided-axis transform as a list of column passes with buffer routing.
bool make_axis_steps(int64_t n, int64_t S, int64_t items, int64_t D, int src, int dst, int spare, int cap,
                     TwiddleBuilder& tb, std::vector<Step>& out, bool& needs_spare)
{
    std::vector<int> fac = split_axis(n, cap);
    if (fac.empty()) return false;
    const int Q = (int)fac.size();
    // routing: pass q reads b[q] and writes b[q+1].  Only the last pass may
    // run in place (its read set equals its write set); every other pass
    // must write a buffer different from the one it reads, and `src` may be
    // reused as scratch only after the first pass consumed it.
    std::vector<int> b(Q + 1);
    b[0] = src;
    b[Q] = dst;
    if (Q >= 2) {
        b[Q - 1] = dst;
        for (int q = Q - 2; q >= 1; --q) b[q] = (b[q + 1] == dst) ? spare : dst;
        if (b[1] == src) {
            if (Q != 2) return false;
            b[1] = spare;
        }
    }
    needs_spare = false;
    int64_t Ns = 1;
    for (int q = 0; q < Q; ++q) {
        Step st;
        if (!make_col_step(n, S, items, D, fac[q], Ns, tb, st)) return false;
        st.src = b[q];
        st.dst = b[q + 1];
        if (st.src == spare || st.dst == spare) needs_spare = true;
        out.push_back(st);
        Ns *= fac[q];
    }
    return true;
}

bool row_feasible(int L, int io_mode)
{
    TwiddleBuilder scratch;
    Step st;
    const bool even = io_mode == IO_R2C_EVEN || io_mode == IO_C2R_EVEN;
    const int64_t in_dist = io_mode == IO_C2R_EVEN ? L + 1 : (io_mode == IO_C2R_ODD ? L / 2 + 1 : L);
    const int64_t out_dist = io_mode == IO_R2C_EVEN ? L + 1 : (io_mode == IO_R2C_ODD ? L / 2 + 1 : L);
    return make_row_step(L, 1, in_dist, out_dist, io_mode, even ? 2 * L : L, WEIGHT_NONE, scratch, st);
}

}  // namespace

std::vector<int> split_axis(int64_t n, int cap)
{
    if (!length_supported(n)) return {};
    if (n <= cap) return {(int)n};
    // smallest number of factors; balanced (closest to n^(1/Q))
    std::vector<int64_t> divs;
    for (int64_t d = 2; d <= cap && d < n; ++d)
        if (n % d == 0) divs.push_back(d);
    for (int Q = 2; Q <= 4; ++Q) {
        const double target = std::pow((double)n, 1.0 / Q);
        std::vector<int> best;
        double best_score = 1e300;
        std::vector<int> cur;
        std::function<void(int64_t, int)> dfs = [&](int64_t rem, int left) {
            if (left == 1) {
                if (rem > cap || rem < 2) return;
                cur.push_back((int)rem);
                double score = 0;
                for (int f : cur) score += std::fabs(std::log((double)f / target));
                if (score < best_score) {
                    best_score = score;
                    best = cur;
                }
                cur.pop_back();
                return;
            }
            for (int64_t d : divs) {
                if (rem % d || rem / d < 2) continue;
                cur.push_back((int)d);
                dfs(rem / d, left - 1);
                cur.pop_back();
            }
        };
        dfs(n, Q);
        if (!best.empty()) {
            // largest factor first: the first pass writes contiguous blocks
            std::sort(best.begin(), best.end(), std::greater<int>());
            return best;
        }
    }
    return {};
}

bool build_scratch_c2c_steps(int64_t n, int64_t batch, TwiddleBuilder& tb, std::vector<Step>& out)
{
    out.clear();
    if (n < 2 || batch < 1 || !length_supported(n)) return false;
    const std::vector<int> fac = split_axis(n, col_max_length());
    if (fac.size() != 2) return false;
    Step first, second;
    if (!make_col_step(n, 1, batch, n, fac[0], 1, tb, first)) return false;
    if (!make_col_step(n, 1, batch, n, fac[1], fac[0], tb, second)) return false;
    first.src = BUF_IN;
    first.dst = BUF_WS;
    second.src = BUF_WS;
    second.dst = BUF_OUT;
    out.push_back(first);
    out.push_back(second);
    return true;
}

namespace {

// One tensor-core pass over sequences q = b*S + s of length L = R*R.
Step tc_step(int L, int prec, int64_t nseq, int64_t S, int64_t in_dist, int64_t in_s, int64_t in_n,
             int64_t out_dist, int64_t out_s, int64_t out_n, int64_t outer_n, TwiddleBuilder& tb)
{
    const int R = L == 256 ? 16 : 8;
    const int TS = 128 / R;
    Step st;
    st.kind = Step::TC;
    TcArgs& a = st.tc;
    a.R = R;
    a.prec = prec;
    a.nseq = nseq;
    a.S = S;
    a.in_dist = in_dist;
    a.in_s = in_s;
    a.in_n = in_n;
    a.out_dist = out_dist;
    a.out_s = out_s;
    a.out_n = out_n;
    a.scale = 1.0f;
    auto mode = [&](int64_t dist, int64_t ss, int64_t sn) {
        // interleaved: side-by-side sequences, whole 16-byte pairs per tile
        if (ss == 1 && S % TS == 0 && nseq % TS == 0 && dist % 2 == 0 && sn % 2 == 0) return (int)TC_IO_INTERLEAVED;
        if (sn == 1 && ss % 2 == 0 && dist % 2 == 0) return (int)TC_IO_CONTIG;
        return (int)TC_IO_GENERIC;
    };
    a.in_mode = mode(in_dist, in_s, in_n);
    a.out_mode = mode(out_dist, out_s, out_n);
    st.bmat_off = tb.add_dft_matrix(R, prec);
    st.tw_off = tb.add_linear(L, L, 1);
    if (outer_n > 1) {
        // W_N^e = hi[e >> sh] * lo[e & mask], e < N
        int sh = 0;
        while ((int64_t(1) << (2 * sh)) < outer_n) ++sh;
        a.otw_shift = sh;
        a.otw_lo_n = 1 << sh;
        a.otw_hi_n = (int)(((outer_n - 1) >> sh) + 1);
        st.hi_off = tb.add_linear(a.otw_hi_n, outer_n, int64_t(1) << sh);
        st.lo_off = tb.add_linear(a.otw_lo_n, outer_n, 1);
    }
    return st;
}

}  // namespace

bool build_tc_c2c_steps(int64_t n, int64_t batch, int prec, bool inplace, TwiddleBuilder& tb, std::vector<Step>& out,
                        int64_t& ws_bytes)
{
    if (prec != TC_PREC_TF32X3 && prec != TC_PREC_BF16X3) return false;
    if (batch < 1) return false;
    const int IN = inplace ? BUF_OUT : BUF_IN;
    ws_bytes = 0;
    out.clear();
    if (n == 64 || n == 256) {
        // one pass: sequence b contiguous; S = batch so every tile is one batch item
        Step st = tc_step((int)n, prec, batch, batch, 0, n, 1, 0, n, 1, 1, tb);
        st.src = IN;
        st.dst = BUF_OUT;
        out.push_back(st);
        return true;
    }
    int64_t L1 = 0;
    for (int64_t c : {int64_t(256), int64_t(64)})
        if (n % c == 0 && (n / c == 64 || n / c == 256)) {
            L1 = c;
            break;
        }
    if (!L1) return false;
    const int64_t L2 = n / L1;  // = S of the first pass
    // pass 1: x[b*n + s + L2*n1] -> W_n^{s*k1} * X1 at ws[b*n + s + L2*k1]
    Step p1 = tc_step((int)L1, prec, batch * L2, L2, n, 1, L2, n, 1, L2, n, tb);
    p1.src = IN;
    p1.dst = BUF_WS;
    // pass 2: ws[b*n + k1*L2 + n2] -> out[b*n + k1 + L1*k2]
    Step p2 = tc_step((int)L2, prec, batch * L1, L1, n, L2, 1, n, 1, L1, 1, tb);
    p2.src = BUF_WS;
    p2.dst = BUF_OUT;
    out.push_back(p1);
    out.push_back(p2);
    ws_bytes = n * batch * 8;
    return true;
}

namespace {

// Element addressing of one side of a double-precision pass (see DPassArgs).
struct DLayout {
    int64_t split = 1, hi = 0, lo = 0, stride = 1;
};

// Double precision: every axis as global-memory Stockham passes
// (csrc/dfft.cu).  A pass never writes the buffer it reads: the passes of an
// axis go src -> WS / WS2 (alternating) -> ... -> OUT, one launch per radix.
bool build_dsteps(const Problem& p, bool inplace, TwiddleBuilder& tb, StepList& out, int64_t& ws_bytes,
                  int64_t& ws2_bytes)
{
    auto unsupported = [&](const char* why) {
        out.supported = false;
        out.why = why;
        return true;
    };
    if (p.weight != WEIGHT_NONE) return unsupported("double precision has no adjoint entries");
    const int IN = inplace ? BUF_OUT : BUF_IN;
    int cur = IN;
    // one axis: ntf transforms of length n; `src` / `dst` the layouts of the
    // first pass's input and the last pass's output, `mid` the layout of the
    // intermediates; io bits of the first and the last pass
    // (in_ws: the last pass writes a workspace instead of the output, for a
    // step that follows; `cur` then names that workspace)
    auto axis = [&](int64_t n, int64_t ntf, DLayout src, DLayout mid, DLayout dst, int io_first, int io_last,
                    bool t_fast, bool in_ws = false) -> bool {
        const std::vector<int> rad = choose_radices((int)n);
        if (rad.empty()) return false;
        const int k = (int)rad.size();
        const int64_t toff = tb.add_dtable(n);
        int from = cur;
        int next_ws = (from == BUF_WS) ? BUF_WS2 : BUF_WS;
        int64_t ns = 1;
        for (int i = 0; i < k; ++i) {
            const bool last = i + 1 == k;
            int to = (last && !in_ws) ? BUF_OUT : next_ws;
            if (last && from == BUF_OUT) to = next_ws;  // a one-pass axis on the output: via a workspace
            Step st;
            st.kind = Step::DPASS;
            DPassArgs& a = st.dp;
            a.ntf = ntf;
            a.n = (int32_t)n;
            a.radix = rad[i];
            a.ns = (int32_t)ns;
            a.io = (i == 0 ? io_first : 0) | (last ? io_last : 0);
            a.t_fast = t_fast ? 1 : 0;
            a.scale = 1.0;
            const DLayout& li = i == 0 ? src : mid;
            const DLayout& lo = (last && to == BUF_OUT) ? dst : mid;
            a.in_split = li.split;
            a.in_hi = li.hi;
            a.in_lo = li.lo;
            a.in_stride = li.stride;
            a.out_split = lo.split;
            a.out_hi = lo.hi;
            a.out_lo = lo.lo;
            a.out_stride = lo.stride;
            st.dtw_off = toff;
            st.src = from;
            st.dst = to;
            out.steps.push_back(st);
            if (to != BUF_OUT) next_ws = (to == BUF_WS) ? BUF_WS2 : BUF_WS;
            from = to;
            ns *= rad[i];
        }
        if (in_ws) {
            cur = from;
            return true;
        }
        if (from != BUF_OUT) {  // the axis ended in a workspace laid out like the output
            Step cp;
            cp.kind = Step::COPY;
            cp.src = from;
            cp.dst = BUF_OUT;
            out.steps.push_back(cp);
        }
        cur = BUF_OUT;
        return true;
    };

    if (p.kind == Kind::C2C) {
        const int nd = p.rank;
        const int64_t dims[3] = {p.n0, nd >= 2 ? p.n1 : 1, nd == 3 ? p.n2 : 1};
        int64_t total = p.batch * std::max<int64_t>(p.stride, 1);
        for (int a = 0; a < nd; ++a) total *= dims[a];
        for (int a = 0; a < nd; ++a)
            if (!length_supported(dims[a])) return unsupported("length has a prime factor > 47");
        for (int a = nd - 1; a >= 0; --a) {
            const int64_t n = dims[a];
            int64_t S = (nd == 1) ? std::max<int64_t>(p.stride, 1) : 1;
            for (int b = a + 1; b < nd; ++b) S *= dims[b];
            if (n == 1) continue;
            DLayout l;
            l.split = S;
            l.hi = n * S;
            l.lo = 1;
            l.stride = S;
            if (!axis(n, total / n, l, l, l, 0, 0, S > 1)) return unsupported("length not decomposable");
        }
        if (out.steps.empty() && IN != BUF_OUT) {
            Step cp;
            cp.kind = Step::COPY;
            cp.src = IN;
            cp.dst = BUF_OUT;
            out.steps.push_back(cp);
        }
        for (Step& s : out.steps)
            if (s.kind == Step::COPY) s.copy_bytes = total * 16;
        ws_bytes = ws2_bytes = total * 16;
        return true;
    }
    if (p.stride > 1) return unsupported("double-precision real transforms are horizontal");
    const bool d2z = p.kind == Kind::R2C;
    const int nd = p.rank;
    const int64_t dims[3] = {p.n0, nd >= 2 ? p.n1 : 1, nd == 3 ? p.n2 : 1};
    const int64_t n = dims[nd - 1], nb = n / 2 + 1;
    int64_t rows = p.batch;  // rows along the fastest axis
    for (int a = 0; a + 1 < nd; ++a) rows *= dims[a];
    for (int a = 0; a < nd; ++a)
        if (!length_supported(dims[a])) return unsupported("length has a prime factor > 47");
    auto need = [&](int64_t a, int64_t b) {
        ws_bytes = std::max(ws_bytes, a);
        ws2_bytes = std::max(ws2_bytes, b);
    };
    // the slower axes: transforms down the columns of the half spectrum,
    // element stride S = the faster axes' extent (the fastest as nb bins)
    auto col_axis = [&](int a, bool in_ws) -> bool {
        int64_t S = nb;
        for (int b = a + 1; b + 1 < nd; ++b) S *= dims[b];
        DLayout l;
        l.split = S;
        l.hi = dims[a] * S;
        l.lo = 1;
        l.stride = S;
        return axis(dims[a], rows * nb / dims[a], l, l, l, 0, 0, true, in_ws);
    };
    if (!d2z) {
        // Z2D: the backward column transforms first, into a workspace
        const size_t c0 = out.steps.size();
        for (int a = nd - 2; a >= 0; --a)
            if (dims[a] > 1 && !col_axis(a, true)) return unsupported("length not decomposable");
        if (out.steps.size() > c0) {
            out.steps[c0].dp.conj_in = 1;
            out.steps.back().dp.conj_out = 1;
            need(rows * nb * 16, rows * nb * 16);
        }
    }
    const int src = cur;  // the input, or the workspace holding the column result
    const int64_t in_bytes = d2z ? rows * n * 8 : rows * nb * 16;
    if (n % 2 == 0) {
        // even N: the real row is an L = N/2 complex row; an L-point
        // transform and the even/odd post-process (D2Z), or the Hermitian
        // pre-process and an L-point transform (Z2D), as in the FP32 path
        const int64_t L = n / 2;
        DLayout rowL;
        rowL.hi = L;
        const int64_t toff = tb.add_dtable(n);  // W_N^k for the pre/post-process
        Step pp;
        pp.kind = Step::DPASS;
        DPassArgs& a = pp.dp;
        a.ntf = rows;
        a.n = (int32_t)n;
        a.radix = 1;
        a.ns = 1;
        a.scale = 1.0;
        a.in_split = a.out_split = 1;
        a.in_stride = a.out_stride = 1;
        pp.dtw_off = toff;
        if (d2z) {
            if (!axis(L, rows, rowL, rowL, rowL, DIO_PAIR_IN, 0, false, true))
                return unsupported("length not decomposable");
            a.io = DIO_R2C_POST;
            a.in_hi = L;
            a.out_hi = nb;
            pp.src = cur;
            pp.dst = BUF_OUT;
            out.steps.push_back(pp);
        } else {
            a.io = DIO_C2R_PRE;
            a.in_hi = nb;
            a.out_hi = L;
            pp.src = src;
            pp.dst = src == BUF_WS2 ? BUF_WS : BUF_WS2;
            out.steps.push_back(pp);
            cur = pp.dst;
            if (!axis(L, rows, rowL, rowL, rowL, 0, DIO_PAIR_OUT, false)) return unsupported("length not decomposable");
            out.steps.back().dp.conj_out = 1;  // the backward transform as a forward one
        }
        need(rows * std::max<int64_t>(L, nb) * 16, rows * std::max<int64_t>(L, nb) * 16);
    } else {
        if (src == BUF_OUT) {
            // in place: input and output rows have different pitches, the
            // input moves to the second workspace first
            Step cp;
            cp.kind = Step::COPY;
            cp.copy_bytes = in_bytes;
            cp.src = BUF_OUT;
            cp.dst = BUF_WS2;
            out.steps.push_back(cp);
            cur = BUF_WS2;
        }
        DLayout full, half, real;
        full.hi = n;
        half.hi = nb;
        real.hi = n;
        if (!axis(n, rows, d2z ? real : half, full, d2z ? half : real, d2z ? DIO_REAL_IN : DIO_HERM_IN,
                  d2z ? DIO_HALF_OUT : DIO_REAL_OUT, false))
            return unsupported("length not decomposable");
        need(rows * n * 16, std::max<int64_t>(rows * n * 16, in_bytes));
    }
    // (the rows start from the input, its copy or the column result in a
    // workspace, never from the output, so their last pass writes the output
    // directly: a copy could not change the row pitch)
    for (const Step& s : out.steps)
        if (s.kind == Step::COPY && s.dst == BUF_OUT) return false;
    if (d2z) {
        // D2Z: the forward column transforms last, over the half spectrum
        cur = BUF_OUT;
        for (int a = nd - 2; a >= 0; --a)
            if (dims[a] > 1 && !col_axis(a, false)) return unsupported("length not decomposable");
        for (Step& s : out.steps)
            if (s.kind == Step::COPY && s.dst == BUF_OUT) s.copy_bytes = rows * nb * 16;
        if (nd > 1) need(rows * nb * 16, rows * nb * 16);
    }
    return true;
}

}  // namespace

bool build_steps(const Problem& p, bool inplace, TwiddleBuilder& tb, StepList& out, int64_t& ws_bytes,
                 int64_t& ws2_bytes)
{
    if (p.dbl) {
        const HintScope hints(&p.hints);
        out = StepList{};
        ws_bytes = 0;
        ws2_bytes = 0;
        return build_dsteps(p, inplace, tb, out, ws_bytes, ws2_bytes);
    }
    const HintScope hints(&p.hints);
    out = StepList{};
    ws_bytes = 0;
    ws2_bytes = 0;
    auto unsupported = [&](const char* why) {
        out.supported = false;
        out.why = why;
        return true;
    };
    const int cap = col_max_length();
    const int IN = inplace ? BUF_OUT : BUF_IN;
    auto need_ws = [&](int64_t bytes) { ws_bytes = std::max(ws_bytes, bytes); };
    auto need_ws2 = [&](int64_t bytes) { ws2_bytes = std::max(ws2_bytes, bytes); };

    if (p.rank == 2 || p.rank == 3) {
        const int nd = p.rank;
        const int64_t dims[3] = {p.n0, p.n1, p.rank == 3 ? p.n2 : 1};
        for (int a = 0; a < nd; ++a)
            if (!length_supported(dims[a])) return unsupported("multi-dimensional length has a prime factor > 47");
        const int64_t last = dims[nd - 1];
        int64_t outer = p.batch;  // rows along the fastest axis
        for (int a = 0; a + 1 < nd; ++a) outer *= dims[a];

        if (p.kind == Kind::C2C) {
            // one transform per axis, fastest first: the first pass reads the
            // input, every later pass works on the output (strided columns)
            const int64_t bytes = outer * last * 8;
            int cur = IN;
            int64_t S = 1;
            for (int a = nd - 1; a >= 0; --a) {
                const int64_t n = dims[a];
                const int64_t items = outer * last / (n * S);
                bool spare = false;
                if (n > 1) {
                    if (S == 1 && n <= row_max_length() && row_feasible((int)n, IO_C2C)) {
                        Step st;
                        if (!make_row_step((int)n, items, n, n, IO_C2C, 0, WEIGHT_NONE, tb, st)) return false;
                        st.src = cur;
                        st.dst = BUF_OUT;
                        out.steps.push_back(st);
                    } else if (!make_axis_steps(n, S, items, n * S, cur, BUF_OUT, BUF_WS, cap, tb, out.steps, spare)) {
                        return unsupported("multi-dimensional axis length not decomposable");
                    }
                    cur = BUF_OUT;
                }
                if (spare) need_ws(bytes);
                S *= n;
            }
            if (out.steps.empty() && IN != BUF_OUT) {  // every length 1: a copy
                Step cp;
                cp.kind = Step::COPY;
                cp.copy_bytes = bytes;
                cp.src = IN;
                cp.dst = BUF_OUT;
                out.steps.push_back(cp);
            }
            return true;
        }

        // real 2D / 3D: rows along the fastest axis through the 1D real
        // planner, the slower axes as column passes over the half spectrum
        // (element stride: the product of the faster axes, the fastest
        // counted as last/2 + 1 bins)
        const int64_t nb = last / 2 + 1;
        const int64_t half_bytes = outer * nb * 8;
        auto col_stride = [&](int a) {
            int64_t S = nb;
            for (int b = a + 1; b + 1 < nd; ++b) S *= dims[b];
            return S;
        };
        auto col_items = [&](int a) {
            int64_t it = p.batch;
            for (int b = 0; b < a; ++b) it *= dims[b];
            return it;
        };
        Problem rows;
        rows.hints = p.hints;
        rows.kind = p.kind;
        rows.n0 = last;
        rows.batch = outer;
        rows.weight = p.weight;
        StepList sub;
        int64_t sub_ws = 0, sub_ws2 = 0;
        bool spare = false;
        if (p.kind == Kind::R2C) {
            if (!build_steps(rows, inplace, tb, sub, sub_ws, sub_ws2)) return false;
            if (!sub.supported) return unsupported(sub.why.c_str());
            out.steps = sub.steps;
            need_ws(sub_ws);
            need_ws2(sub_ws2);
            for (int a = nd - 2; a >= 0; --a) {
                const int64_t n = dims[a], S = col_stride(a);
                if (n == 1) continue;
                if (!make_axis_steps(n, S, col_items(a), n * S, BUF_OUT, BUF_OUT, BUF_WS, cap, tb, out.steps, spare))
                    return unsupported("column length not decomposable");
                if (spare) need_ws(half_bytes);
            }
            return true;
        }
        // C2R: backward column transforms of the half spectrum into the
        // second work area (the input stays intact), then the real rows
        bool cols = false;
        for (int a = 0; a + 1 < nd; ++a) cols |= dims[a] > 1;
        if (!build_steps(rows, cols ? false : inplace, tb, sub, sub_ws, sub_ws2)) return false;
        if (!sub.supported) return unsupported(sub.why.c_str());
        if (cols) {
            int from = IN;
            for (int a = nd - 2; a >= 0; --a) {
                const int64_t n = dims[a], S = col_stride(a);
                if (n == 1) continue;
                if (!make_axis_steps(n, S, col_items(a), n * S, from, BUF_WS2, BUF_WS, cap, tb, out.steps, spare))
                    return unsupported("column length not decomposable");
                if (spare) need_ws(half_bytes);
                from = BUF_WS2;
            }
            out.steps.front().col.conj_in = 1;
            out.steps.back().col.conj_out = 1;
            need_ws2(half_bytes);
            for (Step& s : sub.steps) {
                if (s.src == BUF_WS2 || s.dst == BUF_WS2)
                    return unsupported("C2R rows of this length need a second work area of their own");
                if (s.src == BUF_IN) s.src = BUF_WS2;
            }
        }
        out.steps.insert(out.steps.end(), sub.steps.begin(), sub.steps.end());
        need_ws(sub_ws);
        need_ws2(sub_ws2);
        return true;
    }

    const int64_t N = p.n0;
    if (!length_supported(N)) return unsupported("length has a prime factor > 47");

    if (p.kind == Kind::C2C) {
        if (p.prec != 0 && p.stride == 1) {
            int64_t ws = 0;
            std::vector<Step> tc;
            if (build_tc_c2c_steps(N, p.batch, p.prec, inplace, tb, tc, ws)) {
                out.steps = tc;
                need_ws(ws);
                return true;
            }
        }
        bool spare = false;
        if (p.stride > 1) {
            // VERTICAL: transforms down the columns of [N][stride]
            if (!make_axis_steps(N, p.stride, 1, N * p.stride, IN, BUF_OUT, BUF_WS, cap, tb, out.steps, spare))
                return unsupported("vertical length not decomposable");
            if (spare) need_ws(N * p.stride * 8);
            return true;
        }
        if (cluster_for_batch(N, p.batch)) {
            Step st;
            if (make_cluster_step(N, p.batch, tb, st)) {
                st.src = IN;
                st.dst = BUF_OUT;
                out.steps.push_back(st);
                return true;
            }
        }
        if (N <= row_max_length() && row_feasible((int)N, IO_C2C)) {
            Step st;
            if (!make_row_step((int)N, p.batch, N, N, IO_C2C, 0, WEIGHT_NONE, tb, st)) return false;
            st.src = IN;
            st.dst = BUF_OUT;
            out.steps.push_back(st);
            return true;
        }
        if (!make_axis_steps(N, 1, p.batch, N, IN, BUF_OUT, BUF_WS, cap, tb, out.steps, spare))
            return unsupported("length not decomposable");
        if (spare) need_ws(N * p.batch * 8);
        return true;
    }

    if (p.stride > 1) return unsupported("VERTICAL layout is not supported for R2C/C2R");
    const bool r2c = p.kind == Kind::R2C;
    const int64_t nb = N / 2 + 1;
    const int64_t in_bytes = r2c ? N * p.batch * 4 : nb * p.batch * 8;
    // A single fused kernel reads rows of one pitch and writes rows of
    // another, so an in-place call first copies the input to the workspace.
    auto single = [&](int io_mode, int L, int64_t in_dist, int64_t out_dist) {
        Step st;
        if (!make_row_step(L, p.batch, in_dist, out_dist, io_mode, (int)N, p.weight, tb, st)) return false;
        int src = IN;
        if (inplace) {
            Step cp;
            cp.kind = Step::COPY;
            cp.copy_bytes = in_bytes;
            cp.src = BUF_OUT;
            cp.dst = BUF_WS;
            out.steps.push_back(cp);
            need_ws(in_bytes);
            src = BUF_WS;
        }
        st.src = src;
        st.dst = BUF_OUT;
        out.steps.push_back(st);
        return true;
    };
    if (N % 2 == 0) {
        const int64_t L = N / 2;
        const int mode = r2c ? IO_R2C_EVEN : IO_C2R_EVEN;
        const bool row_ok = L <= row_max_length() && row_feasible((int)L, mode);
        if (row_ok && !cluster_for_batch(L, p.batch)) {
            if (!single(mode, (int)L, r2c ? L : nb, r2c ? nb : L)) return false;
            return true;
        }
        // long real transforms (and short ones in small batches) on a
        // cluster, packing fused (an in-place call first copies the input to
        // the workspace: input and output rows have different pitches)
        {
            Step cl;
            if (cluster_for_batch(L, p.batch) && make_cluster_step(L, p.batch, tb, cl, mode, p.weight)) {
                int src = IN;
                if (inplace) {
                    Step cp;
                    cp.kind = Step::COPY;
                    cp.copy_bytes = in_bytes;
                    cp.src = BUF_OUT;
                    cp.dst = BUF_WS;
                    out.steps.push_back(cp);
                    need_ws(in_bytes);
                    src = BUF_WS;
                }
                cl.src = src;
                cl.dst = BUF_OUT;
                out.steps.push_back(cl);
                return true;
            }
        }
        if (row_ok) return single(mode, (int)L, r2c ? L : nb, r2c ? nb : L);
        // long real transforms: separate packing around a multi-pass C2C
        Step pk;
        pk.kind = Step::PACK;
        pk.pack.L = (int)L;
        pk.pack.ntf = p.batch;
        pk.pack.c2r = r2c ? 0 : 1;
        pk.pack.weight = p.weight;
        pk.pack.scale = 1.f;
        pk.post_off = tb.add_linear(L / 2 + 1, N, 1);
        bool spare = false;
        Step cl;
        const bool use_cluster = make_cluster_step(L, p.batch, tb, cl);
        if (r2c) {
            // input (float2 view) -> ... -> WS, then pack WS -> out
            if (use_cluster) {
                cl.src = IN;
                cl.dst = BUF_WS;
                out.steps.push_back(cl);
            } else if (!make_axis_steps(L, 1, p.batch, L, IN, BUF_WS, BUF_WS2, cap, tb, out.steps, spare)) {
                return unsupported("length not decomposable");
            }
            pk.pack.in_dist = L;
            pk.pack.out_dist = nb;
            pk.src = BUF_WS;
            pk.dst = BUF_OUT;
            out.steps.push_back(pk);
        } else {
            pk.pack.in_dist = nb;
            pk.pack.out_dist = L;
            pk.src = IN;
            pk.dst = BUF_WS;
            out.steps.push_back(pk);
            if (use_cluster) {
                cl.src = BUF_WS;
                cl.dst = BUF_OUT;
                cl.cl.conj_out = 1;
                out.steps.push_back(cl);
            } else {
                if (!make_axis_steps(L, 1, p.batch, L, BUF_WS, BUF_OUT, BUF_WS2, cap, tb, out.steps, spare))
                    return unsupported("length not decomposable");
                out.steps.back().col.conj_out = 1;
            }
        }
        need_ws(L * p.batch * 8);
        if (spare) need_ws2(L * p.batch * 8);
        return true;
    }
    // odd N: full-length complex transform inside one CTA
    const int mode = r2c ? IO_R2C_ODD : IO_C2R_ODD;
    if (N <= row_max_length() && row_feasible((int)N, mode)) {
        if (!single(mode, (int)N, r2c ? N : nb, r2c ? nb : N)) return false;
        return true;
    }
    return unsupported("odd real-data length beyond one CTA");
}

}  // namespace gfft
