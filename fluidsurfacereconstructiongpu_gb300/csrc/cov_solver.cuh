// Covariance accumulation and the G matrix of the anisotropic kernel
// (calculationOfTransformMatricesForParticles, ReconstructionCUDA.cu:
// 689-827), shared by the native and the compatibility kernels.
//
// The covariance is seeded with h^2 I and normalised by the weight sum as
// the reference does; it is accumulated with Kahan compensation.  Its SVD is
// its eigen-decomposition (symmetric positive definite), computed by cyclic
// Jacobi in FP32 and redone in FP64 when the condition number exceeds 1e4.
#pragma once

#include "fsr_common.cuh"

namespace fsr {

#if defined(__CUDACC__)
// Kahan-compensated FP32 accumulator.
struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix (Golub & Van
// Loan, Matrix Computations, sec. 8.5); columns of V are eigenvectors.
template <class T>
__device__ void sym_eig3(T A[3][3], T wv[3], T V[3][3])
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? T(1) : T(0);
    const T tol = sizeof(T) == 4 ? T(1e-14) : T(1e-30);
    for (int sweep = 0; sweep < (sizeof(T) == 4 ? 12 : 24); ++sweep) {
        const T off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        const T dia = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
        if (!(off > tol * dia)) break;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0;
            const int q = pq == 0 ? 1 : 2;
            const T apq = A[p][q];
            if (apq == T(0)) continue;
            const T theta = (A[q][q] - A[p][p]) / (T(2) * apq);
            const T sgn = theta >= T(0) ? T(1) : T(-1);
            const T tt = sgn / (fabs(theta) + sqrt(theta * theta + T(1)));
            const T cs = T(1) / sqrt(tt * tt + T(1));
            const T sn = tt * cs;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const T akp = A[k][p], akq = A[k][q];
                A[k][p] = cs * akp - sn * akq;
                A[k][q] = sn * akp + cs * akq;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const T apk = A[p][k], aqk = A[q][k];
                A[p][k] = cs * apk - sn * aqk;
                A[q][k] = sn * apk + cs * aqk;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const T vkp = V[k][p], vkq = V[k][q];
                V[k][p] = cs * vkp - sn * vkq;
                V[k][q] = sn * vkp + cs * vkq;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) wv[i] = A[i][i];
}

// G = (1/h) cbrt(s1 s2 s3) V diag(1/s) V^T with s = |eigenvalues| clamped
// from below at max(s)/4 (cu:790-822).  Returns the largest support radius
// |r| with |G r| < 1, i.e. smax / cof.
template <class T>
__device__ __forceinline__ float make_G(const T V[3][3], const T w[3], float h_inv, float G[9])
{
    T s0 = fabs(w[0]), s1 = fabs(w[1]), s2 = fabs(w[2]);
    const T smax = fmax(s0, fmax(s1, s2));
    const T lo = smax / T(4);
    s0 = fmax(s0, lo);
    s1 = fmax(s1, lo);
    s2 = fmax(s2, lo);
    const T cof = T(h_inv) * cbrt(s0 * s1 * s2);
    const T inv[3] = {T(1) / s0, T(1) / s1, T(1) / s2};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T acc = T(0);
#pragma unroll
            for (int k = 0; k < 3; ++k) acc += V[i][k] * inv[k] * V[j][k];
            G[3 * i + j] = (float)(acc * cof);
        }
    return (float)(smax / cof);
}


// Weighted covariance sums about the mean: weights w = 1 - (d/R)^3 (wij,
// ReconstructionCUDA.cuh:282-292) for neighbours with d < R.
struct CovAccum {
    Kahan c11, c22, c33, c12, c13, c23, wsum;
    // s = d / R, correctly rounded
    __device__ __forceinline__ void add(float vx, float vy, float vz, float s)
    {
        const float wt = 1.0f - s * s * s;
        wsum.add(wt);
        const float wx = wt * vx, wy = wt * vy;
        c11.add(wx * vx);
        c22.add(wy * vy);
        c33.add(wt * vz * vz);
        c12.add(wx * vy);
        c13.add(wx * vz);
        c23.add(wy * vz);
    }
};

// The same sums with the compensation per chunk instead of per term: each
// term enters a plain FP32 chunk sum (one FMA per entry), and after every
// 32 or more candidates the chunk sums join Kahan-compensated totals.  The
// chunks are short, so their own rounding stays at a few ulps of a chunk,
// and the totals keep the compensation of the per-term form at an eighth of
// its instructions.
struct CovChunkAccum {
    CovAccum tot;
    float w = 0.f, c11 = 0.f, c22 = 0.f, c33 = 0.f, c12 = 0.f, c13 = 0.f, c23 = 0.f;
    __device__ __forceinline__ void add(float vx, float vy, float vz, float s)
    {
        const float wt = 1.0f - s * s * s;
        w += wt;
        const float wx = wt * vx, wy = wt * vy;
        c11 = fmaf(wx, vx, c11);
        c22 = fmaf(wy, vy, c22);
        c33 = fmaf(wt * vz, vz, c33);
        c12 = fmaf(wx, vy, c12);
        c13 = fmaf(wx, vz, c13);
        c23 = fmaf(wy, vz, c23);
    }
    __device__ __forceinline__ void fold()
    {
        tot.wsum.add(w);
        tot.c11.add(c11);
        tot.c22.add(c22);
        tot.c33.add(c33);
        tot.c12.add(c12);
        tot.c13.add(c13);
        tot.c23.add(c23);
        w = c11 = c22 = c33 = c12 = c13 = c23 = 0.f;
    }
};

// G for a particle with nn neighbours within R: I / h for isolated particles
// (fewer than min_neighbors), else (1/h) cbrt(s1 s2 s3) V diag(1/s) V^T with
// the eigenvalues s clamped from below at max(s)/4.  Returns the largest
// support radius |r| with |G r| < 1.  fp64_counter (may be null) counts
// FP64 re-solves.
__device__ __forceinline__ float covariance_to_G(const CovAccum& acc, uint32_t nn, uint32_t min_neighbors, float h,
                                                 float h2, float h_inv, float G[9], uint32_t* fp64_counter)
{
    if (nn < min_neighbors) {
#pragma unroll
        for (int k = 0; k < 9; ++k) G[k] = 0.f;
        G[0] = G[4] = G[8] = h_inv;
        return h;
    }
    const float iw = 1.0f / acc.wsum.s;
    float A[3][3] = {{(h2 + acc.c11.s) * iw, acc.c12.s * iw, acc.c13.s * iw},
                     {acc.c12.s * iw, (h2 + acc.c22.s) * iw, acc.c23.s * iw},
                     {acc.c13.s * iw, acc.c23.s * iw, (h2 + acc.c33.s) * iw}};
    double Ad[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Ad[i][j] = (double)A[i][j];
    float wv[3], V[3][3];
    sym_eig3<float>(A, wv, V);
    const float smax = fmaxf(fabsf(wv[0]), fmaxf(fabsf(wv[1]), fabsf(wv[2])));
    const float smin = fminf(fabsf(wv[0]), fminf(fabsf(wv[1]), fabsf(wv[2])));
    if (!(smin > 0.f) || smax > 1e4f * smin) {
        double wd[3], Vd[3][3];
        sym_eig3<double>(Ad, wd, Vd);
        if (fp64_counter) atomicAdd(fp64_counter, 1u);
        return make_G<double>(Vd, wd, h_inv, G);
    }
    return make_G<float>(V, wv, h_inv, G);
}
#endif

}  // namespace fsr
