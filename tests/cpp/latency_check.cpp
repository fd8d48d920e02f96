// Per-call latency of the drop-in C interface, called from C++ with no interpreter in between:
// the config-0 grid (Simplex at feature scale 50, 64^3 from the origin, seed 1337) through
// fnGenUniformGrid3DDevice + synchronise, fnGenUniformGrid3D into page-locked memory and into a
// std::vector, and fnGenSingle3D; beside them the round trip of a one-byte cudaMemsetAsync +
// synchronise (the floor of any call that waits for the GPU).  Every host output is compared
// with the device output bit for bit; prints the medians and "<n> mismatches".
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

#include "FastNoise/FastNoise_C.h"

template <typename F>
static double median_us(F&& f, int reps)
{
    for (int i = 0; i < 20; ++i) f();
    std::vector<double> t;
    for (int i = 0; i < reps; ++i) {
        const auto t0 = std::chrono::steady_clock::now();
        f();
        t.push_back(std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count());
    }
    std::sort(t.begin(), t.end());
    return t[t.size() / 2];
}

int main()
{
    void* node = fnNewFromMetadata(6, 0);                        // Simplex
    if (!node || !fnSetVariableFloat(node, 0, 50.0f)) { std::printf("setup failed\n"); return 1; }
    const int n = 64 * 64 * 64;
    float* pinned = nullptr;
    float* dev = nullptr;
    float* dmm = nullptr;
    if (cudaMallocHost(&pinned, n * sizeof(float)) != cudaSuccess || cudaMalloc(&dev, n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&dmm, 2 * sizeof(float)) != cudaSuccess) {
        std::printf("allocation failed\n");
        return 1;
    }
    std::vector<float> vec(n, 0.0f), fromdev(n);
    float mm[2];
    const void* nodes[] = {node};
    const int dims[] = {3};
    if (fnJitCompile(nodes, dims, 1) != FN_OK) { std::printf("specialisation failed\n"); return 1; }
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    const double floor_us = median_us([&] { cudaMemsetAsync(dmm, 0, 1, s); cudaStreamSynchronize(s); }, 500);
    const double dev_us = median_us([&] {
        fnGenUniformGrid3DDevice(node, dev, 0, 0, 0, 64, 64, 64, 1, 1, 1, 1337, dmm, s);
        cudaStreamSynchronize(s);
    }, 500);
    const double pinned_us = median_us([&] { fnGenUniformGrid3D(node, pinned, 0, 0, 0, 64, 64, 64, 1, 1, 1, 1337, mm); }, 500);
    const double vec_us = median_us([&] { fnGenUniformGrid3D(node, vec.data(), 0, 0, 0, 64, 64, 64, 1, 1, 1, 1337, mm); }, 500);
    const double single_us = median_us([&] { volatile float v = fnGenSingle3D(node, 1.5f, 2.5f, 3.5f, 7); (void)v; }, 500);
    cudaMemcpy(fromdev.data(), dev, n * sizeof(float), cudaMemcpyDeviceToHost);
    int bad = 0;
    for (int i = 0; i < n; ++i) {
        bad += std::memcmp(&pinned[i], &fromdev[i], 4) != 0;
        bad += std::memcmp(&vec[i], &fromdev[i], 4) != 0;
    }
    std::printf("round trip %.1f us | device call + sync %.1f us | host call: page-locked %.1f us, std::vector %.1f us | "
                "single point %.1f us\n", floor_us, dev_us, pinned_us, vec_us, single_us);
    std::printf("%d mismatches\n", bad);
    fnDeleteNodeRef(node);
    return bad == 0 ? 0 : 1;
}
