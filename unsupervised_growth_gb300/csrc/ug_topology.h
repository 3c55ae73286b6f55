// A generated network topology as the host holds it (ug_topology of the C ABI),
// shared by the device generator (ug_topology.cu) and the directory writer
// (ug_files.cpp).
#pragma once
#include "ugrowth.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

struct ug_topology {
    ug_topology_params params;
    int n_ra = 0, n_i = 0, n_tr = 0;
    double model = 0.0;                          // MODEL_INTERNEURON_DISTANCE
    std::vector<double> ra_xyz, i_xyz;           // 3 per neuron (z = 0 on the square)
    std::vector<int32_t> ri_off, ri_tgt, ir_off, ir_tgt;
    std::vector<double> ri_len, ir_len;          // lengths in microns
    std::vector<int32_t> clustered, random_set;  // the two training arrangements
    int64_t ra_attempts = 0, i_retries = 0;
    int batches = 0;                             // placement batches the device ran
    int64_t launches = 0;                        // kernels launched
    float device_ms = 0.f;                       // device time of the generation
    float stage_ms[3] = {0.f, 0.f, 0.f};         // interneurons, HVC(RA) placement, connections
    int dim() const { return params.arrangement == UG_ARRANGEMENT_SQUARE ? 2 : 3; }
};

// The other translation units' view of a context (ug_host.cu).
void ug_set_last_error(const std::string& msg);
int ug_ctx_device(ug_ctx* ctx);
cudaStream_t ug_ctx_stream(ug_ctx* ctx);
std::recursive_mutex& ug_ctx_mutex(ug_ctx* ctx);
void ug_ctx_add_launches(ug_ctx* ctx, int64_t n);
