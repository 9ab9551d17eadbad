// wcfe_frames.h — what the frame writer (wcfe_vtk.cu) needs from the engine (wcfe_engine.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "wcfe_device.cuh"

namespace wcfe {

// one cell's state as the device holds it, for a frame snapshot
struct FrameSource {
    CellDev dev;                   // device pointers (pos / ea ping-pong; the parity is read on the device)
    int mixed;                     // 1: float-float state layout (WCFE_PREC_MIXED)
    int nv, nt;
    std::vector<int32_t> tri;      // the triangles as the caller gave them (3 nt)
    wcfe_params prm;
    cudaStream_t stream;           // the engine's stream
    int device;
};

// fills `out` for cell `id`; 0 or a WCFE_ERR_* code (message set)
int engine_frame_source(wcfe_engine* e, int32_t id, FrameSource* out);
// the engine's device
int engine_device(wcfe_engine* e);
// sets the calling thread's wcfe_last_error message and returns code
int set_error(const char* msg, int code);

}  // namespace wcfe
