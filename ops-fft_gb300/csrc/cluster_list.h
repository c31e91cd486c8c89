// cluster_list.h - the thread-block-cluster C2C configurations that are built.
// X(id, N, C, Q, P, NT, MINB, Q0, Q1, P0, P1): length N = Q*P split over a
// cluster of C CTAs of NT threads (launch bound NT threads, MINB CTAs per
// SM); the column phase runs Q-point transforms as radix Q0 then Q1, the row
// phase P-point transforms as radix P0 then P1.  The planner takes the first
// entry whose N matches (OPS_FFT_CLUSTER_C=<C> pins the cluster size).
// Lengths that also fit one thread group of a row kernel (N <= 4096) go to
// a cluster only for small batches, where one group per transform would
// leave most SMs idle.
#pragma once
#define GFFT_CLUSTERS(X)                                  \
    X(0, 65536, 16, 256, 256, 256, 2, 16, 16, 16, 16)     \
    X(1, 65536, 8, 256, 256, 512, 1, 16, 16, 16, 16)      \
    X(2, 32768, 8, 128, 256, 256, 2, 16, 8, 16, 16)       \
    X(3, 16384, 8, 128, 128, 128, 3, 16, 8, 16, 8)        \
    X(4, 16384, 4, 128, 128, 256, 2, 16, 8, 16, 8)        \
    X(5, 8192, 4, 64, 128, 128, 3, 8, 8, 16, 8)         \
    X(6, 4096, 4, 64, 64, 128, 5, 8, 8, 8, 8)           \
    X(7, 4096, 8, 64, 64, 64, 8, 8, 8, 8, 8)
#define GFFT_NUM_CLUSTER_CFGS 8
