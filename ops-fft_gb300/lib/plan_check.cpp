// plan_check.cpp - host-side verification of a plan's launches.
//
// Replays the address arithmetic of every kernel launch the plan can make
// (all four call variants) and checks it against the sizes of the buffers
// the launch will receive: user input/output for the call shape, the
// plan's workspaces and its twiddle blob, plus launch-shape limits (threads,
// dynamic shared memory, grid size).  Used by the CPU test-suite so index
// errors are caught without running a kernel.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "handle.h"

namespace {

using namespace gfft;

struct Bufs {
    int64_t bytes[4];  // in, out, ws, ws2
};

bool fail(std::string& why, const std::string& s)
{
    why = s;
    return false;
}

bool check_inner(const InnerPlan& ip, int64_t tw_count, std::string& why)
{
    if (ip.L < 1 || ip.npass < 1 || ip.npass > kMaxPass) return fail(why, "bad inner plan");
    int64_t ns = 1;
    for (int p = 0; p < ip.npass; ++p) {
        const PassDesc& d = ip.pass[p];
        if (d.radix < 1 || d.radix > 47) return fail(why, "bad radix");
        if (d.radix > 16 && ip.rmax != 47) return fail(why, "radix beyond kernel instantiation");
        if (d.ns != ns) return fail(why, "ns mismatch");
        if (ns > 1) {
            if (d.tw_off < 0 || d.tw_off + ns * d.radix > tw_count) return fail(why, "pass twiddle out of table");

            if (ns >= 65536 || ip.L >= 65536) return fail(why, "fast division range exceeded");
            // verify the magic division for every j that occurs
            const int nbf = ip.L / d.radix;
            for (int j = 0; j < nbf; ++j) {
                const unsigned q = (unsigned)(((uint64_t)(unsigned)j * d.ns_magic) >> 32);
                if ((int64_t)q != j / ns) return fail(why, "magic division wrong");
            }
        }
        ns *= d.radix;
    }
    if (ns != ip.L) return fail(why, "radix product != L");
    if (ip.nthr < 1) return fail(why, "no threads");
    return true;
}

// Highest shared buffer (1 = A, 2 = B) that run_passes touches.
int buffers_used(int npass, int start, bool last_global)
{
    int cur = start, used = start;
    for (int p = 0; p < npass; ++p) {
        const int dst = (last_global && p == npass - 1) ? 0 : (cur == 1 ? 2 : 1);
        used = std::max(used, dst);
        cur = dst;
    }
    return used;
}

bool check_row(const Step& s, const Bufs& b, int64_t tw_count, std::string& why)
{
    const RowArgs& a = s.row;
    if (!check_inner(a.ip, tw_count, why)) return false;
    const int L = a.ip.L;
    const int maxthr = a.ip.rmax == 16 ? 512 : 256;
    if (a.codelet < 0 && (a.ip.nthr * a.tfpc > maxthr || a.tfpc < 1)) return fail(why, "row threads");
    if (a.tfpc < 1) return fail(why, "row tile");
    if (a.nstage < 1 || a.nstage > 4) return fail(why, "row stages");
    if (a.codelet >= 0) {
        int cl = 0, cn = 0, cr[kMaxPass], cnr = 0, cmaxt = 0, cminb = 0;
        if (gfft_codelet_info(a.codelet, &cl, &cn, cr, &cnr, &cmaxt, &cminb) != 0 || cl != L || cn != a.ip.nthr ||
            cnr != a.ip.npass)
            return fail(why, "codelet mismatch");
        for (int p = 0; p < cnr; ++p)
            if (cr[p] != a.ip.pass[p].radix) return fail(why, "codelet radix mismatch");
        if (a.nbuf != 1 && a.nbuf != 2) return fail(why, "codelet buffers");
        bool need_tw = false;
        for (int p = 0; p < a.ip.npass; ++p) need_tw |= a.ip.pass[p].ns > 1;
        if (need_tw && a.tw_cnt == 0) return fail(why, "codelet twiddles not in shared memory");
        const int ps = (cr[0] % 2 == 0) ? 4 : 30;
        if (a.pshift != ps) return fail(why, "codelet padding");
    }
    const bool even = a.io_mode == IO_R2C_EVEN || a.io_mode == IO_C2R_EVEN;
    const int maxidx = even ? L : L - 1;
    if (maxidx + (maxidx >> a.pshift) >= a.lpad) return fail(why, "row lpad too small");
    const int64_t row_bytes = a.in_dist * a.in_esize;
    if ((int64_t)a.tfpc * row_bytes > a.stage_bytes || a.stage_bytes % 16) return fail(why, "row stage too small");
    if (a.codelet >= 0) {
        int64_t slots_end = 64 + (int64_t)a.nstage * a.stage_bytes;
        if (a.nbuf == 2) {  // work buffer after the slots, 16-byte aligned, lpad float2
            if (a.smem_work < slots_end || a.smem_work % 16) return fail(why, "codelet work buffer");
            slots_end = a.smem_work + (int64_t)a.lpad * 8;
        }
        if (a.stage_bytes < a.in_dist * a.in_esize + 32 || a.stage_bytes < 16 + (int64_t)a.lpad * 8 || a.tfpc != 1)
            return fail(why, "codelet slot too small");
        int cl = 0, cn = 0, cr[kMaxPass], cnr = 0, cmaxt = 0, cminb = 0;
        gfft_codelet_info(a.codelet, &cl, &cn, cr, &cnr, &cmaxt, &cminb);
        if (a.ngroups < 1 || a.ngroups > 15 || a.ngroups * a.ip.nthr > cmaxt) return fail(why, "codelet groups");
        // tables arrive as 16-byte aligned supersets: one spare unit each
        const int64_t tw_need = a.tw_cnt > 0 ? (int64_t)a.tw_cnt * 8 + 16 : 0;
        const int64_t post_need = a.post_cnt > 0 ? (int64_t)a.post_cnt * 8 + 16 : 0;
        if (a.smem_tw < 128 || a.smem_tw % 16 || a.smem_post % 16 || a.smem_post < a.smem_tw + tw_need ||
            a.smem_stage < a.smem_post + post_need || a.smem_stage % 128 || a.group_bytes % 128 ||
            a.stage_bytes % 16 || slots_end > a.group_bytes ||
            a.smem_bytes < a.smem_stage + (int64_t)a.ngroups * a.group_bytes || a.smem_bytes > kMaxSmemBytes)
            return fail(why, "codelet shared-memory layout");
    } else if (a.smem_tw < 128 || a.smem_post < a.smem_tw + (int64_t)a.tw_cnt * 8 ||
        a.smem_stage < a.smem_post + (int64_t)a.post_cnt * 8 || a.smem_stage % 16 ||
        a.smem_work < a.smem_stage + (int64_t)a.nstage * a.stage_bytes ||
        a.smem_bytes < a.smem_work + (int64_t)a.tfpc * a.nbuf * a.lpad * 8 || a.smem_bytes > kMaxSmemBytes)
        return fail(why, "row shared-memory layout");
    if (a.tw_cnt > 0) {
        for (int p = 0; p < a.ip.npass; ++p) {
            const PassDesc& d = a.ip.pass[p];
            if (d.ns > 1 && (d.tw_off < a.tw_lo || d.tw_off + (int64_t)d.ns * d.radix > a.tw_lo + a.tw_cnt))
                return fail(why, "pass table outside the shared window");
        }
        if (a.tw_lo + (int64_t)a.tw_cnt > tw_count || a.tw_lo % 2) return fail(why, "twiddle window");
    }
    if (a.codelet < 0) {
        const int start = a.io_mode == IO_C2R_EVEN ? 1 : 0;
        const bool last_global = !(a.io_mode == IO_R2C_EVEN || (a.io_mode == IO_C2C && a.staged));
        if (buffers_used(a.ip.npass, start, last_global) > a.nbuf) return fail(why, "row needs more shared buffers");
    }
    if (a.staged && (int64_t)a.tfpc * (L + 1) >= (1 << 22)) return fail(why, "staged copy index range");
    int64_t in_last = 0, out_last = 0, in_es = 8, out_es = 8;
    const int N = a.nreal;
    switch (a.io_mode) {
    case IO_C2C: in_last = L - 1; out_last = L - 1; break;
    case IO_R2C_EVEN: in_last = L - 1; out_last = L; break;
    case IO_C2R_EVEN: in_last = L; out_last = L - 1; break;
    case IO_R2C_ODD: in_es = 4; in_last = N - 1; out_last = N / 2; break;
    case IO_C2R_ODD: in_last = N / 2; out_es = 4; out_last = N - 1; break;
    default: return fail(why, "io mode");
    }
    if (in_es != a.in_esize || in_last + 1 != a.in_dist) return fail(why, "row input layout");
    if (((a.ntf - 1) * a.in_dist + in_last + 1) * in_es > b.bytes[s.src]) return fail(why, "row input out of bounds");
    if (((a.ntf - 1) * a.out_dist + out_last + 1) * out_es > b.bytes[s.dst]) return fail(why, "row output out of bounds");
    if (even && (s.post_off < 0 || s.post_off + L / 2 + 1 > tw_count)) return fail(why, "post twiddle out of table");
    if (even && a.post_cnt != L / 2 + 1) return fail(why, "post twiddle count");
    return true;
}

int64_t max_part(int64_t cpi, int64_t split, int64_t hi, int64_t lo)
{
    const int64_t jmax = cpi - 1;
    return (jmax / split) * hi + std::min(split - 1, jmax) * lo;
}

bool check_col(const Step& s, const Bufs& b, int64_t tw_count, std::string& why)
{
    const ColArgs& a = s.col;
    if (!check_inner(a.ip, tw_count, why)) return false;
    const int L = a.ip.L;
    if (a.codelet >= 0) {
        // column-tile codelet: the codelet's compile-time spec must match the plan
        int cl = 0, cn = 0, cr[kMaxPass], cnr = 0, cmaxt = 0, cminb = 0;
        if (gfft_codelet_info(a.codelet, &cl, &cn, cr, &cnr, &cmaxt, &cminb) != 0 || cl != L)
            return fail(why, "coltile codelet id");
        if (cn != a.ip.nthr || cnr != a.ip.npass) return fail(why, "coltile spec");
        for (int q = 0; q < cnr; ++q)
            if (cr[q] != a.ip.pass[q].radix) return fail(why, "coltile radices");
        if (a.tfpc < 1 || a.tfpc * cn > cmaxt) return fail(why, "coltile threads");
        const int pshift = (cr[0] % 2 == 0) ? 4 : 30;
        const int64_t need = (int64_t)(L - 1) + ((int64_t)(L - 1) >> pshift) + 1;
        if (a.wsize < need) return fail(why, "coltile column region");
        const int64_t tw_bytes = ((int64_t)a.tw_cnt * 8 + 127) & ~(int64_t)127;
        if (tw_bytes + (int64_t)a.tfpc * a.wsize * 8 > a.smem_bytes || a.smem_bytes > kMaxSmemBytes)
            return fail(why, "coltile smem");
        if (a.tw_cnt < 0 || a.tw_lo < 0 || a.tw_lo + (int64_t)a.tw_cnt > tw_count) return fail(why, "coltile tw window");
        for (int q = 0; q < a.ip.npass; ++q)
            if (a.ip.pass[q].ns > 1 && a.tw_cnt > 0 &&
                (a.ip.pass[q].tw_off < a.tw_lo ||
                 a.ip.pass[q].tw_off + (int64_t)a.ip.pass[q].ns * a.ip.pass[q].radix > (int64_t)a.tw_lo + a.tw_cnt))
                return fail(why, "coltile tw window misses a pass table");
        if (a.ons > 1 || a.staged_out) return fail(why, "coltile with outer twiddles or staged output");
    } else {
        const int maxthr = a.ip.rmax == 16 ? 512 : 256;
        if (a.ip.nthr * a.tfpc > maxthr || a.tfpc < 1 || a.tfp < a.tfpc) return fail(why, "col threads");
        if ((int64_t)a.nbuf * L * a.tfp * 8 > kMaxSmemBytes) return fail(why, "col smem");
        if (buffers_used(a.ip.npass, 0, !a.staged_out) > a.nbuf) return fail(why, "col needs more shared buffers");
    }
    if ((a.ncols + a.tfpc - 1) / a.tfpc > 0x7fffffff) return fail(why, "col grid");
    if (a.cpi < 1 || a.ncols % a.cpi != 0) return fail(why, "col cpi");
    const int64_t items = a.ncols / a.cpi;
    const int64_t in_max = (items - 1) * a.in_dist + max_part(a.cpi, a.in_split, a.in_hi, a.in_lo) +
                           (int64_t)(L - 1) * a.in_stride;
    if ((in_max + 1) * 8 > b.bytes[s.src]) return fail(why, "col input out of bounds");
    int64_t out_max;
    if (a.staged_out) {
        out_max = a.ncols * L - 1;
    } else {
        out_max = (items - 1) * a.out_dist + max_part(a.cpi, a.out_split, a.out_hi, a.out_lo) +
                  (int64_t)(L - 1) * a.out_stride;
    }
    if ((out_max + 1) * 8 > b.bytes[s.dst]) return fail(why, "col output out of bounds");
    if (a.ons > 1) {
        const int64_t M = a.ons * L;
        if (M >= (int64_t(1) << 32)) return fail(why, "outer twiddle index overflow");
        const int64_t S = int64_t(1) << a.otw_shift;
        if (s.lo_off < 0 || s.lo_off + S > tw_count) return fail(why, "outer lo table");
        if (s.hi_off < 0 || s.hi_off + (M + S - 1) / S > tw_count) return fail(why, "outer hi table");
        if (a.tw_div < 1) return fail(why, "tw_div");
    }
    return true;
}

bool check_pack(const Step& s, const Bufs& b, int64_t tw_count, std::string& why)
{
    const PackArgs& a = s.pack;
    const int64_t L = a.L;
    const int64_t in_last = a.c2r ? L : L - 1, out_last = a.c2r ? L - 1 : L;
    if (((a.ntf - 1) * a.in_dist + in_last + 1) * 8 > b.bytes[s.src]) return fail(why, "pack input out of bounds");
    if (((a.ntf - 1) * a.out_dist + out_last + 1) * 8 > b.bytes[s.dst]) return fail(why, "pack output out of bounds");
    if (s.post_off < 0 || s.post_off + L / 2 + 1 > tw_count) return fail(why, "pack twiddles");
    return true;
}

}  // namespace

namespace {

// Tensor-core pass: every tile's HBM accesses, 16-byte alignment of the
// vector modes, the batch item shared by a tile and the table ranges.
bool check_tc(const Step& s, const Bufs& b, int64_t tw_count, std::string& why)
{
    const TcArgs& a = s.tc;
    if (a.R != 8 && a.R != 16) return fail(why, "tc radix");
    if (a.prec != TC_PREC_TF32X3 && a.prec != TC_PREC_BF16X3) return fail(why, "tc precision");
    const int64_t L = (int64_t)a.R * a.R, TS = 128 / a.R;
    if (a.nseq < 1 || a.S < 1) return fail(why, "tc sizes");
    if (a.S % TS != 0 && a.S < a.nseq) return fail(why, "tc tile spans two batch items");
    const int64_t ein = b.bytes[s.src] / 8, eout = b.bytes[s.dst] / 8;
    auto mode_ok = [&](int mode, int64_t dist, int64_t ss, int64_t sn) {
        if (mode == TC_IO_INTERLEAVED)
            return ss == 1 && dist % 2 == 0 && sn % 2 == 0 && a.S % TS == 0 && a.nseq % TS == 0;
        if (mode == TC_IO_CONTIG) return sn == 1 && dist % 2 == 0 && ss % 2 == 0;
        return mode == TC_IO_GENERIC;
    };
    if (!mode_ok(a.in_mode, a.in_dist, a.in_s, a.in_n)) return fail(why, "tc input mode");
    if (!mode_ok(a.out_mode, a.out_dist, a.out_s, a.out_n)) return fail(why, "tc output mode");
    if (a.in_dist < 0 || a.in_s < 0 || a.in_n < 0 || a.out_dist < 0 || a.out_s < 0 || a.out_n < 0)
        return fail(why, "tc negative stride");
    const int64_t ntiles = (a.nseq + TS - 1) / TS;
    for (int64_t t = 0; t < ntiles; ++t) {
        const int64_t q0 = t * TS;
        const int64_t nv = std::min<int64_t>(TS, a.nseq - q0);
        const int64_t bi = q0 / a.S, s0 = q0 - bi * a.S;
        if ((q0 + nv - 1) / a.S != bi) return fail(why, "tc tile spans two batch items");
        const int64_t hi_in = bi * a.in_dist + (s0 + nv - 1) * a.in_s + (L - 1) * a.in_n;
        const int64_t hi_out = bi * a.out_dist + (s0 + nv - 1) * a.out_s + (L - 1) * a.out_n;
        if (hi_in >= ein) return fail(why, "tc load out of bounds");
        if (hi_out >= eout) return fail(why, "tc store out of bounds");
        if (a.in_mode == TC_IO_INTERLEAVED && (s0 % 2 != 0 || nv != TS)) return fail(why, "tc interleaved tile");
        if (a.out_mode == TC_IO_INTERLEAVED && (s0 % 2 != 0 || nv != TS)) return fail(why, "tc interleaved tile");
    }
    if (s.bmat_off < 0 || s.bmat_off % 2 || s.bmat_off + gfft_tc_bmat_entries(a.R, a.prec) > tw_count)
        return fail(why, "tc matrix images out of table");
    if (s.tw_off < 0 || s.tw_off + L > tw_count) return fail(why, "tc twiddles out of table");
    if (s.hi_off >= 0) {
        if (s.lo_off < 0 || a.otw_shift < 0 || a.otw_shift > 20) return fail(why, "tc outer twiddle");
        if (s.hi_off + a.otw_hi_n > tw_count || s.lo_off + a.otw_lo_n > tw_count)
            return fail(why, "tc outer twiddle out of table");
        const int64_t emax = (a.S - 1) * (L - 1);
        if ((emax >> a.otw_shift) >= a.otw_hi_n || a.otw_lo_n != (1 << a.otw_shift))
            return fail(why, "tc outer twiddle index range");
    }
    return true;
}

// Cluster transform: the configuration matches the length, every HBM
// access of the column loads and row stores, the twiddle ranges and the
// receive-buffer offsets of the distributed shared-memory stores.
// Double-precision pass: radix and stage consistent, table inside the blob,
// every element read and written inside its buffer.
bool check_dpass(const Step& s, const Bufs& b, int64_t tw_count, std::string& why)
{
    const DPassArgs& a = s.dp;
    if (a.n < 1 || a.radix < 1 || a.radix > 47 || a.n % a.radix || a.ns < 1 || (a.n / a.radix) % a.ns)
        return fail(why, "dpass radix");
    if (a.ntf < 1 || a.in_split < 1 || a.out_split < 1 || a.in_stride < 1 || a.out_stride < 1)
        return fail(why, "dpass layout");
    if (s.dtw_off < 0 || s.dtw_off % 2 || s.dtw_off + 2 * (int64_t)a.n > tw_count) return fail(why, "dpass table");
    auto max_base = [&](int64_t split, int64_t hi, int64_t lo) {
        return ((a.ntf - 1) / split) * hi + std::min<int64_t>(split - 1, a.ntf - 1) * lo;
    };
    const bool herm = (a.io & DIO_HERM_IN) != 0, real_in = (a.io & DIO_REAL_IN) != 0;
    const bool half = (a.io & DIO_HALF_OUT) != 0, real_out = (a.io & DIO_REAL_OUT) != 0;
    int64_t in_last = herm ? a.n / 2 : a.n - 1, out_last = half ? a.n / 2 : a.n - 1;
    if (a.io & (DIO_R2C_POST | DIO_C2R_PRE)) {
        // the real-data step of an even N = 2L: rows of L values and of L + 1 bins
        if (a.n % 2 || a.radix != 1 || a.ns != 1 || a.in_split != 1 || a.out_split != 1 || a.in_stride != 1 ||
            a.out_stride != 1)
            return fail(why, "dpass real step layout");
        const bool post = (a.io & DIO_R2C_POST) != 0;
        in_last = post ? a.n / 2 - 1 : a.n / 2;
        out_last = post ? a.n / 2 : a.n / 2 - 1;
    }
    const int64_t in_need = (max_base(a.in_split, a.in_hi, a.in_lo) + in_last * a.in_stride + 1) * (real_in ? 8 : 16);
    const int64_t out_need =
        (max_base(a.out_split, a.out_hi, a.out_lo) + out_last * a.out_stride + 1) * (real_out ? 8 : 16);
    if (in_need > b.bytes[s.src]) return fail(why, "dpass input out of bounds");
    if (out_need > b.bytes[s.dst]) return fail(why, "dpass output out of bounds");
    if (s.src == s.dst) return fail(why, "dpass in place");
    return true;
}

bool check_cluster(const Step& s, const Bufs& b, int64_t tw_count, std::string& why)
{
    const ClusterArgs& a = s.cl;
    const int64_t n = a.length;
    int C = 0, Q = 0, P = 0, Q0 = 0, P0 = 0, nt = 0, smem = 0;
    if (gfft_cluster_lookup(n, a.csize, &C, &Q, &P, &Q0, &P0, &nt, &smem) != a.kid) return fail(why, "cluster config");
    if ((int64_t)Q * P != n || P % C || Q % C) return fail(why, "cluster split");
    if (smem != a.smem_bytes || smem > kMaxSmemBytes) return fail(why, "cluster shared memory");
    if (a.io_mode != IO_C2C && a.io_mode != IO_R2C_EVEN && a.io_mode != IO_C2R_EVEN) return fail(why, "cluster mode");
    // the real modes read (C2R) or write (R2C) bin n as well
    const int64_t in_hi = a.io_mode == IO_C2R_EVEN ? n : n - 1;
    const int64_t out_hi = a.io_mode == IO_R2C_EVEN ? n : n - 1;
    if (a.ntf < 1 || a.in_dist <= in_hi || a.out_dist <= out_hi) return fail(why, "cluster sizes");
    const int64_t ein = b.bytes[s.src] / 8, eout = b.bytes[s.dst] / 8;
    if ((a.ntf - 1) * a.in_dist + in_hi >= ein) return fail(why, "cluster load out of bounds");
    if ((a.ntf - 1) * a.out_dist + out_hi >= eout) return fail(why, "cluster store out of bounds");
    if (a.io_mode != IO_C2C && (a.post_off < 0 || a.post_off + n + 1 > tw_count))
        return fail(why, "cluster packing twiddles out of table");
    if (a.io_mode == IO_R2C_EVEN) {
        // symmetric row ownership: every row k_q lands on exactly one CTA
        // slot, and k_q and Q - k_q on the same CTA
        const int H = Q / C / 2;
        std::vector<int> seen((size_t)Q, 0);
        for (int kq = 0; kq < Q; ++kq) {
            int d, l;
            if (kq == 0) { d = 0; l = 0; }
            else if (kq == Q / 2) { d = 0; l = H; }
            else if (kq < Q / 2) { d = kq / H; l = kq % H; }
            else { d = (Q - kq) / H; l = H + (Q - kq) % H; }
            if (d >= C || l >= Q / C) return fail(why, "cluster r2c row map");
            if (seen[(size_t)(d * (Q / C) + l)]++) return fail(why, "cluster r2c row map not one-to-one");
            const int m = (Q - kq) % Q;
            const int dm = m == 0 ? 0 : (m == Q / 2 ? 0 : (m < Q / 2 ? m / H : (Q - m) / H));
            if (dm != d) return fail(why, "cluster r2c mirror rows split");
        }
    }
    if (a.twq_off < 0 || a.twq_off + Q > tw_count || a.twp_off < 0 || a.twp_off + P > tw_count)
        return fail(why, "cluster pass tables out of table");
    if (a.outer_off < 0 || a.outer_off + n > tw_count) return fail(why, "cluster outer twiddles out of table");
    if ((int64_t)(P - 1) * (Q - 1) >= n) return fail(why, "cluster outer twiddle index");
    const int PC = P / C, QC = Q / C, RP = P + 1;
    for (int rank = 0; rank < C; ++rank)
        for (int kq = 0; kq < Q; ++kq) {
            const int d = kq / QC, kl = kq % QC;
            const int64_t off = (int64_t)kl * RP + rank * PC + (PC - 1);
            if (d >= C || off >= (int64_t)QC * RP) return fail(why, "cluster exchange offset");
        }
    return true;
}

}  // namespace

extern "C" ACLFFT_API int aclfftDebugCheckPlan(aclfftHandle plan, char* msg, int msglen)
{
    auto report = [&](const std::string& s) {
        if (msg && msglen > 0) {
            std::snprintf(msg, (size_t)msglen, "%s", s.c_str());
        }
    };
    if (!plan || !plan->impl) {
        report("no plan");
        return -1;
    }
    PlanImpl* impl = plan->impl;
    const Problem& p = impl->prob;
    // rows along the fastest axis and that axis' length
    int64_t outer = p.batch, last = p.n0;
    if (p.rank == 2) {
        outer *= p.n0;
        last = p.n1;
    } else if (p.rank == 3) {
        outer *= p.n0 * p.n1;
        last = p.n2;
    }
    const int64_t es = p.dbl ? 2 : 1;  // double precision: twice the bytes per element
    const int64_t cbytes = (p.rank == 1 ? p.batch * p.n0 * std::max<int64_t>(p.stride, 1) * 8 : outer * last * 8) * es;
    const int64_t rbytes = outer * last * 4 * es;
    const int64_t hbytes = outer * (last / 2 + 1) * 8 * es;
    for (int v = 0; v < 4; ++v) {
        const StepList& sl = impl->lists[v];
        if (!sl.supported) continue;
        Bufs b{};
        int64_t in_b = cbytes, out_b = cbytes;
        const bool adj = v >= 2;
        if (p.kind == Kind::R2C) {
            in_b = adj ? hbytes : rbytes;
            out_b = adj ? rbytes : hbytes;
        } else if (p.kind == Kind::C2R) {
            in_b = adj ? rbytes : hbytes;
            out_b = adj ? hbytes : rbytes;
        }
        const bool inplace = (v & 1) != 0;
        b.bytes[0] = inplace ? 0 : in_b;
        b.bytes[1] = inplace ? std::max(in_b, out_b) : out_b;
        b.bytes[2] = impl->ws_bytes;
        b.bytes[3] = impl->ws2_bytes;
        for (size_t i = 0; i < sl.steps.size(); ++i) {
            const Step& s = sl.steps[i];
            std::string why;
            bool ok = true;
            if (s.src < 0 || s.src > 3 || s.dst < 0 || s.dst > 3) ok = fail(why, "buffer id");
            else if (s.kind == Step::ROW) ok = check_row(s, b, impl->tb.count, why);
            else if (s.kind == Step::COL) ok = check_col(s, b, impl->tb.count, why);
            else if (s.kind == Step::PACK) ok = check_pack(s, b, impl->tb.count, why);
            else if (s.kind == Step::TC) ok = check_tc(s, b, impl->tb.count, why);
            else if (s.kind == Step::CLUSTER) ok = check_cluster(s, b, impl->tb.count, why);
            else if (s.kind == Step::DPASS) ok = check_dpass(s, b, impl->tb.count, why);
            else if (s.kind == Step::COPY)
                ok = (s.copy_bytes <= b.bytes[s.src] && s.copy_bytes <= b.bytes[s.dst]) || fail(why, "copy size");
            if (!ok) {
                char buf[160];
                std::snprintf(buf, sizeof(buf), "variant %d step %zu: ", v, i);
                report(buf + why);
                return 1 + v;
            }
        }
    }
    report("ok");
    return 0;
}
