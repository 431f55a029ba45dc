// Shared between the FP64 tandem (mq_tandem.cu) and the mixed-precision tandem engine
// (mq_tandem_mixed.cu): device track arrays and device field pointers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "mq_tandem.h"

namespace mqtm {

struct Tracks64 {   // FP64 track states on the device (the ABI's mq_tracks, device side)
    double *x, *y, *z, *vx, *vy, *vz;
    uint64_t* rng;
    int32_t *sp, *region, *last;
};

struct DevFields {   // device copies of the description's field arrays (float4 per node)
    const float4* crf;
    const float4* cdc[2];
    const float4 *prf[9], *pac[9], *pdc[9], *pgate[9];
};

struct State;   // the mixed engine's device data (packed fields, mixed-precision tracks, lists)

// pack the cube and port fields for the mixed engine; nullptr (and err) on failure
State* create(const mq_tandem_desc& d, const DevFields& f, cudaStream_t st, std::string& err);
void destroy(State* s);
// FP64 device tracks -> the engine's mixed state (n tracks)
cudaError_t load(State* s, const Tracks64& tr, uint32_t n, cudaStream_t st, uint32_t* launches);
// advance the mixed state by k global steps (drive: k x 10 floats, RF + nine tones) starting at
// global step step0; counts (9 x 21 u32) and stepc (3 u64) accumulate on the device
cudaError_t run(State* s, uint32_t n, const float* drive, uint64_t step0, uint64_t k, uint32_t* counts,
                unsigned long long* stepc, cudaStream_t st, uint32_t* launches);
// the engine's mixed state -> FP64 device tracks
cudaError_t store(State* s, const Tracks64& tr, uint32_t n, cudaStream_t st, uint32_t* launches);

}  // namespace mqtm
