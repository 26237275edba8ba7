// tc_kernel_check.cu -- the tensor-core grid-product kernel (decaes_tc.cu)
// on its own, against exact CPU sums: random grid bases in [0, 1] and echo
// trains, a voxel list skipping every 7th voxel, several shapes (4..128
// echoes, FP32 and FP64 images).  Each product must be within 2e-9 of the
// exact sum relative to the sum of the absolute terms, no row may be marked
// unusable and no block may give up a wait.  With arguments "m n K V" it runs
// one larger FP32 case (timing and profiling).  Built and run by
// tests/test_gpu_tc_kernel.py.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <climits>
#include <vector>
#include <random>
#include "decaes_tc.h"
// the library's shared-memory limit helper (decaes_gpu.cu), for this driver alone
namespace dh {
int raise_smem_limit(const void *kern, size_t bytes) {
    return (int)cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
}
#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("CUDA %s at %d: %s\n", #x, __LINE__, cudaGetErrorString(e)); exit(2);} } while (0)
int run(int m, int n, int K, long V, bool f32, int sms, int reps) {
    std::mt19937_64 g(m * 1000 + n);
    std::uniform_real_distribution<double> U(0, 1);
    std::vector<double> As((size_t)K * m * n);
    for (auto &a : As) a = U(g);
    std::vector<double> img((size_t)V * m);
    for (auto &y : img) y = 2000 * U(g) + 1;
    std::vector<int> vidx;
    for (long v = 0; v < V; ++v) if (v % 7 != 3) vidx.push_back((int)v);
    int nv = (int)vidx.size();
    const int mpad = dk::tc_mpad(m), ntiles = dk::tc_ntiles(K, n);
    const long ldF = 2L * ntiles * dk::kTcTileN;
    double *dAs; void *dimg; int *dvidx, *dnv, *dFexp; unsigned *derr; float *dF; unsigned char *dB;
    size_t bbytes = (size_t)ntiles * dk::kTcSlices * dk::tc_slice_bytes(dk::kTcTileN, mpad);
    CK(cudaMalloc(&dAs, sizeof(double) * As.size()));
    CK(cudaMemcpy(dAs, As.data(), sizeof(double) * As.size(), cudaMemcpyHostToDevice));
    std::vector<float> imgf(img.begin(), img.end());
    if (f32) for (size_t i = 0; i < img.size(); ++i) img[i] = imgf[i];
    CK(cudaMalloc(&dimg, (f32 ? 4 : 8) * img.size()));
    if (f32) CK(cudaMemcpy(dimg, imgf.data(), 4 * img.size(), cudaMemcpyHostToDevice));
    else CK(cudaMemcpy(dimg, img.data(), 8 * img.size(), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&dvidx, 4 * nv)); CK(cudaMemcpy(dvidx, vidx.data(), 4 * nv, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&dnv, 4)); CK(cudaMemcpy(dnv, &nv, 4, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&dFexp, 4 * (size_t)nv)); CK(cudaMalloc(&derr, 4)); CK(cudaMemset(derr, 0, 4));
    CK(cudaMalloc(&dF, 4 * (size_t)nv * ldF)); CK(cudaMalloc(&dB, bbytes));
    CK(dk::tc_make_basis_slices(dAs, m, n, K, dB, 0));
    dk::TcParams p{};
    p.image = dimg; p.f32 = f32; p.V = V; p.m = m; p.mpad = mpad; p.vidx = dvidx; p.nvox = dnv; p.t0 = 0; p.t1 = nv;
    p.Bsl = dB; p.ntiles = ntiles; p.F = dF; p.ldF = ldF; p.Fexp = dFexp; p.err = derr;
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    for (int r = 0; r < reps; ++r) {
        if (r == reps - 1) cudaEventRecord(e0);
        CK(dk::tc_grid_products(p, sms, 0));
        if (r == reps - 1) cudaEventRecord(e1);
    }
    CK(cudaDeviceSynchronize());
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    std::vector<float> F((size_t)nv * ldF); std::vector<int> Fexp(nv); unsigned err;
    CK(cudaMemcpy(F.data(), dF, 4 * F.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(Fexp.data(), dFexp, 4 * nv, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&err, derr, 4, cudaMemcpyDeviceToHost));
    double mr = 0; long bad = 0;
    long check = std::min<long>(nv, 4000);
    for (int t = 0; t < check; ++t) {
        long v = vidx[t];
        if (Fexp[t] == INT_MIN) { bad++; continue; }
        double sc = std::ldexp(1.0, Fexp[t]);
        for (int k = 0; k < K; ++k) for (int j = 0; j < n; ++j) {
            double ex = 0, ab = 0;
            for (int i = 0; i < m; ++i) { double q = As[(size_t)k * m * n + i + (size_t)m * j] * img[v + V * i]; ex += q; ab += std::fabs(q); }
            double got = ((double)F[(size_t)t * ldF + 2 * (k * n + j)] + (double)F[(size_t)t * ldF + 2 * (k * n + j) + 1]) * sc;
            double r = std::fabs(got - ex) / ab;
            if (r > mr) mr = r;
        }
    }
    double bytes = (double)nv * (ldF * 4.0 + 4.0 + 4.0 * m);
    printf("m=%d n=%d K=%d V=%ld f32=%d: voxels %d, unusable %ld, err %u, max rel %.3g, %.3f ms, %.0f GB/s\n",
           m, n, K, V, (int)f32, nv, bad, err, mr, ms, bytes / (ms * 1e-3) / 1e9);
    cudaFree(dAs); cudaFree(dimg); cudaFree(dvidx); cudaFree(dnv); cudaFree(dFexp); cudaFree(derr); cudaFree(dF); cudaFree(dB);
    return (bad == 0 && err == 0 && mr < 2e-9) ? 0 : 1;
}
int main(int argc, char **argv) {
    int sms = 0; CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
    int rc = 0;
    if (argc > 1) {  // one large case (timing / profiling): m n K V
        rc |= run(atoi(argv[1]), atoi(argv[2]), atoi(argv[3]), atol(argv[4]), true, sms, 3);
    } else {
        rc |= run(48, 40, 32, 1000, true, sms, 1);
        rc |= run(48, 40, 32, 3000, false, sms, 1);
        rc |= run(56, 60, 64, 700, true, sms, 1);
        rc |= run(24, 48, 8, 500, false, sms, 1);
        rc |= run(128, 64, 4, 300, true, sms, 1);
        rc |= run(4, 2, 2, 50, false, sms, 1);
    }
    printf(rc ? "FAIL\n" : "PASS\n");
    return rc;
}
