// Host launchers of the tcgen05 MLP kernels (pjg_mlp.cu).
#pragma once
#include <cstdint>

int mlp_launch_rows(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int N, int K,
                 const float* bias, int act, const void* zp, int64_t ldzp, void* Y, int64_t ldy,
                 void* YT, int64_t ldyt, void* Z, int64_t ldz, float* Y32, int64_t ldy32,
                 float* colsum, void* stream);
int mlp_launch_wgrad(const void* A, int64_t lda, const void* B, int64_t ldb, int Mo, int No, int64_t Kb,
                  float* C, int64_t ldc, void* stream);
int mlp_launch_fused(const void* X, int64_t ldx, int64_t M, const void* const* W,
                     const float* const* b, float* Y, int64_t ldy, void* stream);
int surr_launch_features(int64_t n, int nn, const double* phi, const double* param,
                         const double* st, void* X, float floor_c, void* stream);
int surr_launch_outputs(int64_t n, int nn, const float* Y, const double* phi, const double* param,
                        const double* st, int err_col, double* dphi, float* lerr, void* stream);
int mlp_error_flag(int clear);
