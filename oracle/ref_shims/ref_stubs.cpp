// Link stubs for oracle/ref_harness.cpp.  The reference's host code refers to
// CUDA helper functions and to GPU stage classes whose definitions live in
// .cu files the CPU harness does not build.  The CPU path never calls them;
// each stub aborts if it is ever reached.  Test infrastructure only.
#include <cstdio>
#include <cstdlib>
#include <string>
#include "CudaUtils.cuh"
#include "KernelUtilsFactory.h"

namespace CudaUtils {
cudaDeviceProp deviceProp;
size_t getTotalMemory() { return (size_t)1 << 50; }
size_t getUsedMemory() { return 0; }
}

[[noreturn]] static void gpu_stub(const char* what) {
  std::fprintf(stderr, "reference GPU stage reached in CPU harness: %s\n", what);
  std::abort();
}

template <> void AddSurfacesAlgorithm_GPU_CUDA<float, float>::performAddSurfaces(
    CellGrid<float>*, CellGrid<float>*, CellGrid<float>*) { gpu_stub("AddSurfaces"); }
template <> void RemoveNegativeElevationsAlgorithm_GPU_CUDA<float>::performRemoveNegativeElevationValues(
    CellGrid<float>*) { gpu_stub("RemoveNegativeElevations"); }
