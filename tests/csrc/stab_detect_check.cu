// Test harness (not part of the library): runs the engine's stability-limit
// detector in its one-lane form, its lane-parallel form and its
// mixed-precision form on the same scaled-derivative histories and returns
// the three results.
#include "amici_gb300/csrc/engine.cuh"

__global__ void stab_detect_check(const double* hist, const int* q, int n, int* seq, int* par, int* mix) {
    const int h = blockIdx.x;  // one history per warp
    if (h >= n) return;
    const double* ss = hist + (size_t)h * 15;
    const int lane = threadIdx.x & 31;
    const int r_par = agb::sl_detect_group<32>(ss, q[h], 0xffffffffu, lane);
    const int r_mix = agb::sl_detect_mixed<32>(ss, q[h], 0xffffffffu, lane);
    if (lane == 0) {
        par[h] = r_par;
        mix[h] = r_mix;
        seq[h] = agb::sl_detect(ss, q[h]);
    }
}

extern "C" int run_stab_detect_check(const double* hist, const int* q, int n, int* seq, int* par, int* mix) {
    double* dh;
    int *dq, *ds, *dp, *dm;
    cudaMalloc(&dh, sizeof(double) * 15 * n);
    cudaMalloc(&dq, sizeof(int) * n);
    cudaMalloc(&ds, sizeof(int) * n);
    cudaMalloc(&dp, sizeof(int) * n);
    cudaMalloc(&dm, sizeof(int) * n);
    cudaMemcpy(dh, hist, sizeof(double) * 15 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dq, q, sizeof(int) * n, cudaMemcpyHostToDevice);
    stab_detect_check<<<n, 32>>>(dh, dq, n, ds, dp, dm);
    cudaError_t e = cudaDeviceSynchronize();
    cudaMemcpy(seq, ds, sizeof(int) * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(par, dp, sizeof(int) * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(mix, dm, sizeof(int) * n, cudaMemcpyDeviceToHost);
    cudaFree(dh);
    cudaFree(dq);
    cudaFree(ds);
    cudaFree(dp);
    cudaFree(dm);
    return (int)e;
}
