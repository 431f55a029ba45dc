// Bounds checks of the debug build.  Compiled with -DMQ_CHECK (build(check=True) makes
// libmqgb_check.so), every gather whose index is computed from a particle's position, and the
// work-queue indices of the persistent kernels, go through MQ_CHK / MQ_CHK_SPAN: an index out of
// range is recorded (count, site, index, limit) in a per-translation-unit device word and
// replaced by 0, so the access stays inside the array and the kernel runs on; the host reads the
// words with mq_check_status.  In the normal build the macros are the bare index.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

struct MqCheckWord {
    unsigned int hits;         // out-of-range indices seen
    unsigned int site;         // site id of the first one
    unsigned long long index;  // its index (or first element of its span)
    unsigned long long limit;  // the array length it was checked against
};

#ifdef MQ_CHECK
static __device__ MqCheckWord g_mq_check;

__device__ __forceinline__ void mq_chk_record(size_t i, size_t n, unsigned site) {
    if (atomicAdd(&g_mq_check.hits, 1u) == 0u) {
        g_mq_check.site = site;
        g_mq_check.index = i;
        g_mq_check.limit = n;
    }
}
// i must lie in [0, n)
__device__ __forceinline__ size_t mq_chk(size_t i, size_t n, unsigned site) {
    if (i < n) return i;
    mq_chk_record(i, n, site);
    return 0;
}
// elements [i, i + span) must lie in [0, n)
__device__ __forceinline__ size_t mq_chk_span(size_t i, size_t span, size_t n, unsigned site) {
    if (i + span <= n && i + span >= i) return i;
    mq_chk_record(i, n, site);
    return 0;
}
#define MQ_CHK(i, n, site) mq_chk((size_t)(i), (size_t)(n), (site))
#define MQ_CHK_SPAN(i, span, n, site) mq_chk_span((size_t)(i), (size_t)(span), (size_t)(n), (site))
// host reader of this translation unit's word: 0 = read (and cleared when reset != 0)
#define MQ_CHECK_READER(fn)                                                                          \
    extern "C" int fn(MqCheckWord* out, int reset) {                                                 \
        if (cudaMemcpyFromSymbol(out, g_mq_check, sizeof(MqCheckWord)) != cudaSuccess) {             \
            cudaGetLastError();                                                                      \
            return -2;                                                                               \
        }                                                                                            \
        if (reset) {                                                                                 \
            const MqCheckWord z = {0u, 0u, 0ull, 0ull};                                              \
            if (cudaMemcpyToSymbol(g_mq_check, &z, sizeof(z)) != cudaSuccess) {                      \
                cudaGetLastError();                                                                  \
                return -2;                                                                           \
            }                                                                                        \
        }                                                                                            \
        return 0;                                                                                    \
    }
#else
#define MQ_CHK(i, n, site) (i)
#define MQ_CHK_SPAN(i, span, n, site) (i)
#define MQ_CHECK_READER(fn)                                                                          \
    extern "C" int fn(MqCheckWord* out, int reset) {                                                 \
        (void)reset;                                                                                 \
        out->hits = 0u; out->site = 0u; out->index = 0ull; out->limit = 0ull;                        \
        return 1;                                                                                    \
    }
#endif

// site ids
enum MqCheckSite : unsigned {
    MQ_SITE_F64_FIELD = 1, MQ_SITE_F64_CRASH = 2,
    MQ_SITE_MIX_CELL = 10, MQ_SITE_MIX_ION = 11, MQ_SITE_MIX_LIST_OUT = 12,
    MQ_SITE_TDM_CUBE = 20, MQ_SITE_TDM_PORT = 21, MQ_SITE_TDM_GATE = 22, MQ_SITE_TDM_CRASH = 23,
    MQ_SITE_TMX_CELL = 30, MQ_SITE_TMX_LIST = 31,
    MQ_SITE_SELFTEST = 99,
};
