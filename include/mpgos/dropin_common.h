// Pieces shared by the two drop-in headers (per-thread and coupled): the
// reference's error macro, its device helper functions
// (SingleSystem_PerThread_Interface.cuh:67-69 and
// CoupledSystems_PerBlock_Interface.cuh:73-75 declare the same three) and the
// status-to-exit mapping of the drop-in classes.
#ifndef MPGOS_DROPIN_COMMON_H
#define MPGOS_DROPIN_COMMON_H

#include <cuda_runtime.h>
#include <stdio.h>

#include <cstdlib>
#include <cstring>
#include <iostream>

#include "../mpgos.h"
#include "dropin_print.h"

#define gpuErrCHK(call)                                                                           \
    {                                                                                             \
        const cudaError_t error_ = call;                                                          \
        if (error_ != cudaSuccess) {                                                              \
            std::cout << "Error: " << __FILE__ << ":" << __LINE__ << std::endl;                   \
            std::cout << "code:" << error_ << ", reason: " << cudaGetErrorString(error_) << std::endl; \
            exit(1);                                                                              \
        }                                                                                         \
    }

// ---- device helpers --------------------------------------------------------
inline void PrintPropertiesOfSpecificDevice(int device)
{
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) {
        std::cerr << "ERROR: cannot query device " << device << std::endl;
        exit(EXIT_FAILURE);
    }
    int clock_khz = 0, mem_clock_khz = 0;
    cudaDeviceGetAttribute(&clock_khz, cudaDevAttrClockRate, device);
    cudaDeviceGetAttribute(&mem_clock_khz, cudaDevAttrMemoryClockRate, device);
    std::cout << "Device number: " << device << std::endl;
    std::cout << "Device name:   " << p.name << std::endl;
    std::cout << "--------------------------------------" << std::endl;
    std::cout << "Total global memory:        " << p.totalGlobalMem / 1024 / 1024 << " Mb" << std::endl;
    std::cout << "Total shared memory:        " << p.sharedMemPerBlock / 1024 << " Kb" << std::endl;
    std::cout << "Number of 32-bit registers: " << p.regsPerBlock << std::endl;
    std::cout << "Number of multiprocessors:  " << p.multiProcessorCount << std::endl;
    std::cout << "Compute capability:         " << p.major << "." << p.minor << std::endl;
    std::cout << "Core clock rate:            " << clock_khz / 1000 << " MHz" << std::endl;
    std::cout << "Memory clock rate:          " << mem_clock_khz / 1000 << " MHz" << std::endl;
    std::cout << "Memory bus width:           " << p.memoryBusWidth << " bits" << std::endl;
    std::cout << "Warp size:                  " << p.warpSize << std::endl;
    std::cout << "Max. threads per multiproc: " << p.maxThreadsPerMultiProcessor << std::endl;
    std::cout << "Max. threads per block:     " << p.maxThreadsPerBlock << std::endl << std::endl;
}

inline void ListCUDADevices()
{
    int n = 0;
    cudaGetDeviceCount(&n);
    for (int i = 0; i < n; i++) PrintPropertiesOfSpecificDevice(i);
}

inline int SelectDeviceByClosestRevision(int major, int minor)
{
    cudaDeviceProp want;
    std::memset(&want, 0, sizeof(want));
    want.major = major;
    want.minor = minor;
    int device = 0;
    cudaChooseDevice(&device, &want);
    std::cout << "CUDA Device Number Closest to Revision " << major << "." << minor << ": " << device << std::endl;
    return device;
}

namespace mpgos {
namespace dropin {
inline void check(int rc, const char* what)
{
    if (rc != MPGOS_OK) {
        std::cerr << "ERROR: In solver member function " << what << "!" << std::endl;
        std::cerr << "       " << mpgos_last_error() << std::endl;
        exit(EXIT_FAILURE);
    }
}
inline void bound(const char* fn, const char* what, int value, int lo, int hi)
{
    if (value < lo || value > hi) {
        std::cerr << "ERROR: In solver member function " << fn << "!" << std::endl;
        std::cerr << "       Option: " << what << std::endl;
        if (lo > hi)
            std::cerr << "       Acceptable index: none" << std::endl;
        else
            std::cerr << "       Acceptable index: " << lo << "-" << hi << std::endl;
        std::cerr << "       Current index:    " << value << std::endl;
        exit(EXIT_FAILURE);
    }
}
}  // namespace dropin
}  // namespace mpgos

#endif
