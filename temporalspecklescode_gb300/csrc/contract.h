// contract.h -- launch interface of the contraction kernels (contract.cu, gemm_tc.cu).
#pragma once
#include <cuda_runtime.h>

#include "scene.h"

namespace sstmc {

// V[t][v][l] += sum_{p < K} A[p][t][l] * B[p][t][v]  (times W[t][v][l] if W),
// restricted to rows with mat[p] == mat_sel when mat is given.
struct GemmParams {
    const float2* A;
    const float2* B;
    int K, Nt, Nl, Nv;
    const unsigned char* mat;
    int mat_sel;
    const float* W;
    double2* V;
    int kchunk;
    int compensated;
    int* err;             // tensor-core form: SSTMC_TIMEOUT if a bounded wait ran out
    int real;             // tensor-core form: A, B hold real floats [K][Nt][Nl] / [K][Nt][Nv] (V gets the real part)
    double scale;         // V += scale * sum (field CBS: 1 / sqrt(2)); 0 reads as 1
    // tensor-core form, far-field x far-field single scattering: rows grouped by
    // material, one launch for every material of mats[0 .. nmat): material m
    // contracts rows bucket[m] .. bucket[m + 1] with the weights W + m * wstride
    const uint32_t* bucket;   // [kMat + 1] on the device, or null
    int nmat;
    int mats[kMat];
    size_t wstride;
};

// Stable partition of a chunk's n paths by the material of their first vertex:
// ss_row[q] = the path's row, bucket[m] .. bucket[m + 1] = material m's rows.
struct SsBucketParams {
    const float4* verts;
    const uint32_t* counts;
    const uint32_t* offsets;
    uint32_t n, nblocks;
    uint32_t* hist;       // [ceil(n / 1024)][kMat] scratch
    uint32_t* ss_row;     // [n]
    uint32_t* bucket;     // [kMat + 1]
};
int launch_ss_buckets(const SsBucketParams& P, cudaStream_t stream);

// V[t][v][l] += sum_p a[p][t][l] * b[p][t][v] * W(l, v, t, p), W from the
// scatterer position x1[p] / x1t[p][t] and material m1[p].
struct SsParams {
    const float2* a;
    const float2* b;
    const float* x1;
    const float* x1t;
    const unsigned char* m1;
    int K;
    double2* V;
    int kchunk;
    int compensated;
};

int launch_gemm(const GemmParams& G, cudaStream_t stream);
// tcgen05 3xTF32 form of launch_gemm (gemm_tc.cu); chooses its own K split.
bool gemm_tc_eligible(const GemmParams& G);
int launch_gemm_tc(const GemmParams& G, cudaStream_t stream);
int launch_ss(const DevScene& S, const SsParams& G, cudaStream_t stream);

}  // namespace sstmc
