// wcfe_serving.h — what the serving loop (wcfe_server.cu) needs from the engine
// (wcfe_engine.cu): cells prepared on host threads, admitted and retired in stream
// order without a host synchronisation, and stepped with a device-side step budget.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/wcfe.h"
#include "wcfe_topology.h"

namespace wcfe {

// A request's cell as the host prepares it before admission: connectivity, patches, the
// derived static arrays and the start state in the engine's layout, and the exact device
// bytes it will take.  Built by serving_prepare without any CUDA call (thread-safe).
struct PreparedCell {
    Topology topo;
    Patches patches;
    wcfe_params prm{};
    int32_t steps = 0;               // the step budget of the cell (ctl[3])
    int32_t nk1 = 0;
    size_t soff[32] = {}, poff[7] = {};
    size_t state_bytes = 0, patch_bytes = 0;
    std::vector<int4> tri4, patch_tri;
    std::vector<int32_t> bnd_vert;
    std::vector<double> ca;          // c_A = 100 in the engine's layout
    std::vector<double> pos;         // start positions in the engine's layout (4 doubles per vertex)
    bool mixed = false;
};

// Host-only preparation of a cell for engine e (its precision and patch shape); "" or an error.
std::string serving_prepare(const wcfe_engine* e, PreparedCell& pc, int32_t nv, int32_t nt, const int32_t* tri,
                            const double* x, const wcfe_params& prm, int32_t steps);
// Allocate the cell's blocks from `pool` on stream st, upload it on st and add it to the
// engine (not yet synchronised: the caller makes the engine stream wait for st).  The
// prepared arrays must stay alive until st has run the copies.  0 or a WCFE_ERR_* code.
int serving_admit(wcfe_engine* e, PreparedCell& pc, cudaStream_t st, cudaMemPool_t pool, int32_t* id);
// Enqueue nsteps explicit steps of every cell on the engine stream (tables refreshed
// without a host synchronisation); no host wait.
int serving_step(wcfe_engine* e, int32_t nsteps, double dt);
// Enqueue, on the engine stream, the copy of cell id's positions (raw device layout,
// buffer `parity`) into pinned host memory, then free the cell in stream order.
// *bytes receives the size of the raw copy (32 bytes per vertex).
int serving_retire(wcfe_engine* e, int32_t id, int parity, void* pinned_dst, size_t cap, size_t* bytes);
// Raw device positions (as serving_retire copies them) to double[n][3].
void serving_decode_positions(const wcfe_engine* e, const void* raw, int32_t nv, double* x);
size_t serving_raw_bytes(int32_t nv);
cudaStream_t engine_stream(const wcfe_engine* e);
int engine_device(wcfe_engine* e);
uint64_t engine_budget(const wcfe_engine* e);
uint64_t engine_used(const wcfe_engine* e);
int set_error(const char* msg, int code);

}  // namespace wcfe
