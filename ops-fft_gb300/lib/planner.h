// planner.h - plan-time decisions for the GB300 aclfft library.
//
// Pure host code (no CUDA calls), so it is unit-testable without a GPU.
// Responsibilities that the reference defers to every exec call
// (src/fft1_d/arch35/fft/fft1_d_c2c.cpp:82-136,188-239) happen once here:
//   * prime factorisation and the support decision (primes <= 47, the
//     reference's RADIX_MIX set, src/common/host/fft_exec_helper.h:76);
//   * the radix sequence of every on-chip Stockham transform;
//   * the decomposition of long or strided axes into column passes;
//   * the list of twiddle-table segments the GPU generator must fill;
//   * the device workspace size.
#pragma once
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../csrc/kernel_args.h"

namespace gfft {

std::vector<int64_t> prime_factors(int64_t n);  // ascending, with multiplicity
bool all_primes_at_most(int64_t n, int64_t pmax);

// Largest on-chip lengths (complex elements) the generic kernels accept.
int row_max_length();
int col_max_length();

// Compile-time specialised row kernels are used unless OPS_FFT_CODELETS=0.
bool codelets_enabled();

// Long C2C lengths with a cluster configuration run on thread-block
// clusters unless OPS_FFT_CLUSTER=0.
bool clusters_enabled();

// Radix sequence for an on-chip transform of length L (product == L),
// radices <= 16 when possible, primes up to 47 otherwise.  Empty on failure.
std::vector<int> choose_radices(int L);

// Split an axis of length n into on-chip factors, each <= cap.
std::vector<int> split_axis(int64_t n, int cap);

enum BufId : int { BUF_IN = 0, BUF_OUT = 1, BUF_WS = 2, BUF_WS2 = 3 };

struct Step {
    enum Kind { ROW, COL, PACK, COPY, TC, CLUSTER, DPASS } kind = ROW;
    int64_t copy_bytes = 0;
    RowArgs row{};
    ColArgs col{};
    PackArgs pack{};
    TcArgs tc{};
    ClusterArgs cl{};
    DPassArgs dp{};  // double precision
    int src = BUF_IN;
    int dst = BUF_OUT;
    // Offsets (float2 units) into the plan's twiddle blob for the pointers
    // patched at exec time; -1 when unused.
    int64_t tw_off = -1, post_off = -1, hi_off = -1, lo_off = -1;
    int64_t bmat_off = -1;  // TC: DFT-matrix operand images
    int64_t dtw_off = -1;   // DPASS: FP64 table W_n^m (float2 units, 2 per entry)
};

// Everything needed to run one transform kind (forward / adjoint variants
// are separate StepLists).
struct StepList {
    std::vector<Step> steps;
    bool supported = true;
    std::string why;  // reason when unsupported
};

struct TwiddleBuilder {
    std::vector<TwSeg> segs;
    int64_t count = 0;  // float2 entries so far (kept 2-aligned)
    // FP64 tables W_n^m, m < n (double precision plans): (offset, n), each
    // 2n float2 entries of the blob
    std::vector<std::pair<int64_t, int64_t>> dsegs;
    int64_t add_dtable(int64_t n);
    int64_t add_pass_table(int64_t ns, int R);        // rows of R, W_{ns*R}^{k*r}
    int64_t add_linear(int64_t count, int64_t M, int64_t mult);  // W_M^{i*mult}
    int64_t add_dft_matrix(int R, int prec);  // tensor-core operand images (kind 3)
};

// Fill ip for length L with the given radices; register tables in tb.
bool build_inner(int L, const std::vector<int>& radices, int nthr, TwiddleBuilder& tb, InnerPlan& ip);

// High-level builder: appends the steps of one transform to `out` and its
// twiddle segments to `tb`.  `inplace` builds the variant used when the
// caller passes the same buffer as input and output.  ws_bytes / ws2_bytes
// receive the device workspace the steps need.
enum class Kind { C2C, R2C, C2R };

// Choices that override the planner's defaults for one plan (the plan
// autotuner sets them; the default values keep the static rules and the
// OPS_FFT_* environment knobs).
struct PlanHints {
    int codelet_variant = -1;  // k-th specialised build of the length
    int codelet_ng = 0;        // transform groups per CTA of a codelet
    int codelet_nst = 0;       // input prefetch stages of a codelet
    int codelet_pp = -1;       // 1: per-group work buffer (ping-pong passes), 0: in place
    int codelets = -1;         // 0: no specialised row kernels
    int cluster = -1;          // 0: no cluster kernels; 1: clusters wherever a configuration exists
    int cluster_c = 0;         // cluster size
    bool operator==(const PlanHints& o) const
    {
        return codelet_variant == o.codelet_variant && codelet_ng == o.codelet_ng && codelet_nst == o.codelet_nst &&
               codelet_pp == o.codelet_pp && codelets == o.codelets && cluster == o.cluster &&
               cluster_c == o.cluster_c;
    }
};

struct Problem {
    PlanHints hints;
    Kind kind = Kind::C2C;
    int rank = 1;
    int64_t n0 = 1, n1 = 1, n2 = 1;  // 1D: n0 = N. 2D: n0 = nx (slow), n1 = ny (fast). 3D: n0, n1, n2 = nx, ny, nz
    int64_t batch = 1;
    int64_t stride = 1;      // VERTICAL 1D: stride between samples (= batch), batch = 1
    int weight = WEIGHT_NONE;
    int prec = 0;            // 0: FP32 Stockham; TcPrec: split-precision tensor-core stages (C2C)
    bool dbl = false;        // double precision (Z2Z / D2Z / Z2D)
};

bool build_steps(const Problem& p, bool inplace, TwiddleBuilder& tb, StepList& out, int64_t& ws_bytes,
                 int64_t& ws2_bytes);

// Two column passes of a long batched C2C (length n = L1 * L2): the first
// writes its whole output to BUF_WS, the second reads BUF_WS and writes
// BUF_OUT.  False when n does not split into exactly two on-chip factors.
bool build_scratch_c2c_steps(int64_t n, int64_t batch, TwiddleBuilder& tb, std::vector<Step>& out);

// Split-precision tensor-core steps of a 1D batched C2C of length n
// (64, 256 or a product of two of them).  False when n has no such split.
bool build_tc_c2c_steps(int64_t n, int64_t batch, int prec, bool inplace, TwiddleBuilder& tb,
                        std::vector<Step>& out, int64_t& ws_bytes);

// Which transform length families are executable (reference domain).
bool length_supported(int64_t n);

}  // namespace gfft
