/*
 * A C caller of the GPU library in the pattern of the reference's driver
 * (lila-c/main_w03.c:129-200): seeded A, the workspace query, one call of
 * lila_dgeqrf_w03_recursive on device buffers, then the library's own
 * checks ||A - QR||_F / ||A||_F and ||I - Q^T Q||_F.  Plain C (C11) against
 * include/lila.h and include/lila_gpu.h: it shows that a reference caller
 * switches by changing its allocations, not its calls.
 *
 *   main_w03_gpu [m n mt nx]     prints one line; exit 0 when rc == 0, the
 *                                status word is clear and both checks are
 *                                at most 50 n 2^-53.
 */
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime.h>

#include "lila.h"
#include "lila_gpu.h"

int main(int argc, char **argv)
{
    int m = argc > 1 ? atoi(argv[1]) : 2000;
    int n = argc > 2 ? atoi(argv[2]) : 300;
    int mt = argc > 3 ? atoi(argv[3]) : 64;
    int nx = argc > 4 ? atoi(argv[4]) : 64;
    int lila_param[4] = {0, 1, 1, nx}; /* leaf 1, panel 1 (lila-c/main_w03.c:150-153) */
    size_t bytes = sizeof(double) * (size_t)m * (size_t)n;
    double *hA = (double *)malloc(bytes);
    double *dA = NULL, *dA0 = NULL, *dT = NULL, *dQ = NULL, *dW = NULL;
    unsigned s = 12345u;
    size_t k;
    int lwork, rc, status;
    double res, orth, tol;

    if (!hA || m < n || n < 1) return 2;
    for (k = 0; k < (size_t)m * (size_t)n; k++) {
        s = s * 1103515245u + 12345u;
        hA[k] = (double)(s >> 8) / 16777216.0 - 0.5;
    }
    if (cudaMalloc((void **)&dA, bytes) != cudaSuccess || cudaMalloc((void **)&dA0, bytes) != cudaSuccess ||
        cudaMalloc((void **)&dQ, bytes) != cudaSuccess ||
        cudaMalloc((void **)&dT, sizeof(double) * (size_t)mt * (size_t)n) != cudaSuccess)
        return 3;
    cudaMemcpy(dA, hA, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dA0, hA, bytes, cudaMemcpyHostToDevice);
    lwork = lila_query_dgeqrf_w03_recursive(lila_param, m, n, 0, mt, NULL, m, NULL, mt, NULL, m, NULL, -1);
    if (cudaMalloc((void **)&dW, sizeof(double) * (size_t)lwork) != cudaSuccess) return 3;

    rc = lila_dgeqrf_w03_recursive(lila_param, m, n, 0, mt, dA, m, dT, mt, dQ, m, dW, lwork);
    lila_gpu_sync();
    status = lila_gpu_status();
    orth = lila_test_qq_orth_1(m, n, 0, dQ, m);
    res = lila_test_qr_repres_1(m, n, 0, dA0, m, dQ, m, dA, m);
    tol = 50.0 * n * 1.1102230246251565e-16;
    printf("m %d n %d mt %d nx %d rc %d status %d res %.3e orth %.3e tol %.3e\n", m, n, mt, nx, rc, status, res,
           orth, tol);
    cudaFree(dA);
    cudaFree(dA0);
    cudaFree(dQ);
    cudaFree(dT);
    cudaFree(dW);
    free(hA);
    return (rc == 0 && status == 0 && res <= tol && orth <= tol) ? 0 : 1;
}
