// Allocation-free FP64 stepping for callers that cannot allocate device memory (see the
// comment on mq_run_ions_device_noalloc in include/mq_engine.h).
//
// The FP64 step kernel needs two pieces of working memory besides the caller's inputs and
// outputs: the per-job constant table and a pair of counters (executed steps, live ions).
// Here both live in one file-scope static device array.  Host code never uses the array's
// name as an address (on the host it only names a stand-in object): the device address is
// looked up with cudaGetSymbolAddress with the device current, once per device and CUDA
// context (a reset device gets a new context, and the address is looked up again), and that
// pointer is what the kernels receive.
#include <cuda.h>

#include <mutex>

#include "mq_engine.h"
#include "mq_internal.h"

namespace {

constexpr size_t kCounterBytes = 256;   // [0] u64 executed steps, [8] u32 live ions, [12] u32 bad job indices
static_assert(sizeof(mqp::JobC) == 96, "scratch sizing assumes a 96-byte job record");
static_assert(MQ_NOALLOC_SCRATCH_BYTES == kCounterBytes + MQ_NOALLOC_MAX_JOBS * sizeof(mqp::JobC), "scratch layout");

// The scratch: counters, then MQ_NOALLOC_MAX_JOBS job records.  Every GPU that loads the
// library holds these 393,472 bytes until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[MQ_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
struct Slot {
    unsigned long long ctx = 0;   // id of the context the address belongs to (0 = none)
    void* addr = nullptr;
};
Slot g_slot[kMaxDevices];

typedef CUresult (*ctx_get_current_fn)(CUcontext*);
typedef CUresult (*ctx_get_id_fn)(CUcontext, unsigned long long*);

// id of the calling thread's current context (unique per context the process creates), or 0
// when the driver does not report one; looked up through the runtime's driver entry points so
// the library needs no link against the driver library
unsigned long long current_context_id() {
    static ctx_get_current_fn get_current = nullptr;
    static ctx_get_id_fn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<ctx_get_current_fn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<ctx_get_id_fn>(p);
        cudaGetLastError();
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// device address of the scratch on device `dev`, which the caller has made current: looked up
// once per device and context (every call when the driver reports no context id)
cudaError_t scratch_address(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lk(g_lock);
    const unsigned long long ctx = current_context_id();
    Slot& s = g_slot[dev];
    if (!s.addr || ctx == 0 || s.ctx != ctx) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        s.addr = p;
        s.ctx = ctx;
    }
    *out = static_cast<unsigned char*>(s.addr);
    return cudaSuccess;
}

// counts the ions whose job index is not below njobs (the step kernel reads the job table at
// that index without a check)
__global__ void k_count_bad_jid(const uint32_t* __restrict__ jid, uint32_t n, uint32_t njobs, uint32_t* bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool b = i < n && jid[i] >= njobs;
    const unsigned m = __ballot_sync(0xffffffffu, b);
    if (m && (threadIdx.x & 31) == (unsigned)(__ffs(m) - 1)) atomicAdd(bad, (uint32_t)__popc(m));
}

constexpr uint32_t kChunk = 50000;   // steps per launch, as the FP64 engine
constexpr size_t kStage = 128;       // job records converted per host-side batch (stack buffer)

}  // namespace

extern "C" mq_status mq_run_ions_device_noalloc(const mq_dev_grid* grid, const mq_job* jobs, size_t njobs,
                                                const mq_physics* ph, const mq_ions* io, size_t n, uint32_t max_more,
                                                void* stream, uint64_t* ion_steps) {
    if (ion_steps) *ion_steps = 0;
    if (!grid || !jobs || !ph || !io || njobs == 0 || !grid->rf4 || !grid->ac4 || !grid->dc4) return MQ_ERR_INVALID;
    if (grid->nx < 3 || grid->ny < 3 || grid->nz < 3 || !(grid->h > 0)) return MQ_ERR_INVALID;
    if (njobs > MQ_NOALLOC_MAX_JOBS) return MQ_ERR_TOO_LARGE;      // fixed scratch: at most 4096 jobs
    if (n > 0xFFFFFFF0ull) return MQ_ERR_TOO_LARGE;
    const char* why = nullptr;   // the species, physics and shared-RF checks of every other entry point
    const mq_status chk = mqd::check_jobs(jobs, njobs, ph, &why);
    if (chk != MQ_OK) return chk;
    if (!io->x || !io->y || !io->z || !io->vx || !io->vy || !io->vz || !io->ph_rf || !io->ph_ac || !io->rng ||
        !io->steps || !io->ncoll || !io->leg || !io->status || !io->jid)
        return MQ_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MQ_ERR_NO_DEVICE;
    if (cudaSetDevice(dev) != cudaSuccess) return MQ_ERR_NO_DEVICE;   // makes the device's context current
    unsigned char* base = nullptr;
    if (scratch_address(dev, &base) != cudaSuccess) return MQ_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long* d_steps = reinterpret_cast<unsigned long long*>(base);
    uint32_t* d_live = reinterpret_cast<uint32_t*>(base + 8);
    uint32_t* d_bad = reinterpret_cast<uint32_t*>(base + 12);
    mqp::JobC* d_jobs = reinterpret_cast<mqp::JobC*>(base + kCounterBytes);

    // every ion's job index must name one of the jobs: the states are device memory, so the check
    // runs on the device before anything is written
    if (n > 0) {
        if (cudaMemsetAsync(d_bad, 0, 4, st) != cudaSuccess) return MQ_ERR_CUDA;
        k_count_bad_jid<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(io->jid, (uint32_t)n, (uint32_t)njobs, d_bad);
        if (cudaGetLastError() != cudaSuccess) return MQ_ERR_CUDA;
        uint32_t bad = 0;
        if (cudaMemcpyAsync(&bad, d_bad, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return MQ_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return MQ_ERR_CUDA;
        if (bad != 0) return MQ_ERR_INVALID;
    }
    // job constants, converted on the host in small stack batches and copied into the scratch
    for (size_t k0 = 0; k0 < njobs; k0 += kStage) {
        mqp::JobC buf[kStage];
        const size_t m = njobs - k0 < kStage ? njobs - k0 : kStage;
        for (size_t k = 0; k < m; ++k) buf[k] = mqd::host_job(jobs[k0 + k], *ph);
        // from pageable memory this copy returns once buf has been read, so buf may be reused
        if (cudaMemcpyAsync(d_jobs + k0, buf, m * sizeof(mqp::JobC), cudaMemcpyHostToDevice, st) != cudaSuccess)
            return MQ_ERR_CUDA;
    }
    const mqp::Batch b = mqd::host_batch(grid->nx, grid->ny, grid->nz, grid->h, grid->axis_mm, grid->layers_mm, *ph,
                                         jobs[0].drive);
    mqd::DevGrid g;
    g.rf = reinterpret_cast<const float4*>(grid->rf4);
    g.ac = reinterpret_cast<const float4*>(grid->ac4);
    g.dc = reinterpret_cast<const float4*>(grid->dc4);
    g.nx = grid->nx; g.ny = grid->ny; g.nz = grid->nz; g.pad = 0; g.h = grid->h; g.inv_h = 1.0 / grid->h;
    mqd::DevIons d;
    d.x = io->x; d.y = io->y; d.z = io->z; d.vx = io->vx; d.vy = io->vy; d.vz = io->vz;
    d.ph_rf = io->ph_rf; d.ph_ac = io->ph_ac; d.rng = io->rng; d.steps = io->steps; d.ncoll = io->ncoll;
    d.leg = io->leg; d.status = io->status; d.jid = io->jid;

    if (cudaMemsetAsync(d_steps, 0, 8, st) != cudaSuccess) return MQ_ERR_CUDA;   // the scratch keeps old values
    uint64_t budget = max_more;
    for (;;) {
        const uint32_t L = budget < kChunk ? (uint32_t)budget : kChunk;
        if (L == 0) break;
        if (cudaMemsetAsync(d_live, 0, 4, st) != cudaSuccess) return MQ_ERR_CUDA;
        // no phase tables (length 0): the kernel evaluates every drive phase directly
        if (mqd::launch_f64_step(g, b, d_jobs, nullptr, nullptr, 0, d, (uint32_t)n, L, d_steps, d_live, st) != cudaSuccess)
            return MQ_ERR_CUDA;
        uint32_t live = 0;
        if (cudaMemcpyAsync(&live, d_live, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return MQ_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return MQ_ERR_CUDA;
        budget -= L;
        if (live == 0) break;
    }
    unsigned long long steps = 0;
    if (cudaMemcpyAsync(&steps, d_steps, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return MQ_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MQ_ERR_CUDA;
    if (ion_steps) *ion_steps = steps;
    return MQ_OK;
}
