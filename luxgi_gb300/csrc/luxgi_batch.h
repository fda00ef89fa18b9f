// Batched launches of many volumes: the plan a frame of a volume set runs
// (shared by the batch objects and the serving loop).
#pragma once

#include <vector>

#include "luxgi_volume.h"

namespace luxgi {

// block-offset tables of the batched launches; kWork holds each volume's
// first batch-wide march work index instead
enum Stage { kRaygen, kWeights, kMarch, kShade, kBlendI, kBlendD, kWork, kPack, kNumStages };

// What a set of volumes needs to run one frame as batched launches.
struct Plan {
    std::vector<luxgi_ddgi_volume*> vols;
    luxgi_ddgi_batch_tuning t{};
    int n = 0;
    int storage = 0, light_mode = 0, sdf_format = 0;
    bool tc = false;
    // per-frame argument block: TraceParams[n], BlendParams[n], then the
    // tensor-core jobs (tc_bytes a volume, 128-byte aligned)
    size_t off_trace = 0, off_blend = 0, off_tc = 0, tc_bytes = 0, arg_bytes = 0;
    std::vector<int> starts;            // [kNumStages][n + 1] block offsets
    int blocks[kNumStages] = {};
    size_t smem_i = 0, smem_d = 0;      // dynamic shared memory of the FP32 blend
    std::vector<TcPlan> tcp;            // tensor-core blend maps, one per volume
    TcLaunch tcl;                       // the one tensor-core blend launch of the frame
    // march compaction shared by the plan's volumes (budget 0: one pass)
    int budget = 0;
    int64_t work = 0;                   // march work items of all volumes
    uint32_t qa_cap = 0, qb_cap = 0;
    int4* q = nullptr;                  // device queues + counters (plan_set_aux)
    uint32_t* qcount = nullptr;
    // shading in bin order over the whole batch (sorted false: march order)
    bool sorted = false;
    uint32_t* sbins = nullptr;          // [2][kBatchShadeBins]
    uint2* skeys = nullptr;             // [work] (bin, rank) of each batch-wide work item
    uint32_t* sseq = nullptr;           // [work] batch-wide work items by bin
};

// Device bytes of the plan's march queues and shading-order arrays, and
// binding them to a device region of that size (16-byte aligned).
size_t plan_aux_bytes(const Plan& P);
void plan_set_aux(Plan& P, void* dev);

int compat_check(luxgi_ddgi_volume* const* vols, int n);
bool tuning_valid(const luxgi_ddgi_batch_tuning& t);
luxgi_ddgi_batch_tuning default_tuning();
// Gives every volume the plan's march and shade variant (packed SDF copies follow).
int apply_variants(luxgi_ddgi_volume* const* vols, int n, const luxgi_ddgi_batch_tuning& t);
int plan_build(Plan& P, luxgi_ddgi_volume* const* vols, int n, const luxgi_ddgi_batch_tuning& t);
// Per-frame arguments of every volume in its current state (P.arg_bytes).
void plan_fill(const Plan& P, const float* rots, uint8_t* host);
// One frame: d_args holds plan_fill's block, d_starts the plan's tables.
cudaError_t plan_launch(const Plan& P, uint8_t* d_args, const int* d_starts, cudaStream_t st);
int prepare_all(const Plan& P, cudaStream_t st);
void end_frame_all(const Plan& P);

}  // namespace luxgi
