// Internal interface of the whole-path object (pipeline.cu), shared with the request server (server.cu).
#pragma once
#include "cs_common.cuh"

#include <memory>

namespace csg
{

enum Stage
{
    ST_KEYS,
    ST_SORT,
    ST_GATHER,
    ST_BUILD,
    ST_LINK,
    ST_GEO,
    ST_NBPREP,
    ST_HALOS,
    ST_NEIGHBORS,
    ST_COUNT
};

struct PipelineBase
{
    cs_pipeline_config cfg{};
    virtual ~PipelineBase() = default;
    virtual int run(cudaStream_t s, const void* x, const void* y, const void* z, const void* h, size_t n,
                    const cs_box& box, uint64_t f0, uint64_t f1, cs_pipeline_result* res, bool hostIn) = 0;
    virtual int outputs(cs_pipeline_outputs* o) = 0;
    virtual size_t deviceBytes() const          = 0;
    //! enqueue the copy of the last run's counts and halo flags (either may be null) to host memory, and optionally
    //! its neighbour lists as CSR (listOffsets: n + 1 entries; list: listCap entries; both pinned host memory)
    virtual int copyBackAsync(cudaStream_t s, uint32_t* nc, uint8_t* flags, size_t flagsCap,
                              uint64_t* listOffsets = nullptr, uint32_t* list = nullptr, size_t listCap = 0) = 0;
    //! wait for the last copy-back; the first device error of the runs since the previous wait
    virtual int wait() = 0;
    virtual int step(cudaStream_t s, const void* x, const void* y, const void* z, const void* h, size_t n,
                     const cs_box& box, bool useGraph, cs_pipeline_result* res) = 0;
    virtual void resetSteps() = 0;
    //! times the neighbour search of the last run's inputs for each candidate tuning and keeps the fastest
    virtual int autotune(cudaStream_t s, int reps, cs_tuning* best, cs_tuning* tried, float* ms, int capacity,
                         int* count) = 0;
    //! device times of the last copy-back that returned neighbour lists (waits for it): compaction, list copy, the
    //! list copy's wait for its stream, and the run's start to the end of its list copy
    virtual int copyTimes(float* ms, int count) = 0;
    int graphReplays = 0; // steps of the last step sequence that were replayed from a captured graph
    cs_tuning tuning{32, 7, 16};
    cudaEvent_t ev[ST_COUNT + 1] = {};
    float stageMs[ST_COUNT]      = {};
    int lastN                    = 0;
};

//! a pipeline object for the coordinate and key widths (32 or 64 bits each)
std::unique_ptr<PipelineBase> makePipeline(int coordBits, int keyBits, const cs_pipeline_config& cfg);

//! device checksum of a neighbour result: the wrapping sum over particles i of a hash of (i, count, the first
//! min(count, ngmax) stored indices); order-independent over particles, so equal results give equal sums
uint64_t neighborChecksum(cudaStream_t s, const uint32_t* nb, const uint32_t* nc, size_t n, unsigned ngmax,
                          uint64_t* scratchDev);

} // namespace csg
