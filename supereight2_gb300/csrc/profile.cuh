// profile.cuh — RAII event pairs around kernel launches (see profile.cu).
#pragma once

#include "se_gpu_internal.cuh"

namespace se_gpu {

enum {
    kProfBeginFrame = 0,
    kProfCarve,
    kProfFrustum,
    kProfUpdate,
    kProfRaycast,
    kProfTrackPrep,
    kProfIcpIter,
    kProfIcpCheck,
    kProfFrameGraph, // a whole captured frame (graph launch)
    kProfCount
};

// Event pairs cannot be recorded into a graph under capture: capture code suspends profiling.
void profiling_suspend(bool suspend);

class ProfScope {
  public:
    ProfScope(int kernel, cudaStream_t stream);
    ~ProfScope();
    ProfScope(const ProfScope&) = delete;
    ProfScope& operator=(const ProfScope&) = delete;

  private:
    int kernel_;
    cudaStream_t stream_;
    cudaEvent_t start_;
};

} // namespace se_gpu
