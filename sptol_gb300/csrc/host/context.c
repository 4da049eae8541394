/*
 * Library context: device selection, the library stream, launch counting,
 * the thread-local last-error slot (same contract as the reference's
 * src/error/error.c:28-116) and timers (include/includes/helper_funcs.h:42-48).
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "../sptgb_internal.h"
#include "../../../include/sptgb.h"

static pthread_once_t g_once = PTHREAD_ONCE_INIT;
static int g_init_err = 0;
static int g_device = 0;
static cudaStream_t g_stream = NULL;
static cudaStream_t g_copy_stream = NULL;   /* host-buffer uploads that overlap device work on g_stream */
static _Atomic uint64_t g_launches = 0;
static uint64_t g_seed = 0x5eed5eedULL;
static int g_quiet = -1;

static __thread struct {
    const char *module;
    int errcode;
    const char *file;
    unsigned line;
    char *reason;
} g_last = {NULL, 0, NULL, 0, NULL};

int sptgb_quiet(void) {
    if (g_quiet < 0) {
        const char *q = getenv("SPTGB_QUIET");
        g_quiet = (q && q[0] && q[0] != '0') ? 1 : 0;
    }
    return g_quiet;
}

void spt_ComplainError(const char *module, int errcode, const char *file, unsigned line, const char *reason) {
    g_last.errcode = errcode;
    g_last.module = module;
    g_last.file = file;
    g_last.line = line;
    if (reason) {
        free(g_last.reason);
        g_last.reason = strdup(reason);
    }
    if (!sptgb_quiet()) {
        if (g_last.reason && g_last.reason[0])
            fprintf(stderr, "[%s] error 0x%08x at %s:%u, %s\n", module, errcode, file, line, g_last.reason);
        else
            fprintf(stderr, "[%s] error 0x%08x at %s:%u\n", module, errcode, file, line);
    }
}

int sptGetLastError(const char **module, const char **file, unsigned *line, const char **reason) {
    if (module) *module = g_last.module;
    if (file) *file = g_last.file;
    if (line) *line = g_last.line;
    if (reason) *reason = g_last.reason;
    return g_last.errcode;
}

void sptClearLastError(void) {
    g_last.module = NULL;
    g_last.errcode = 0;
    g_last.file = NULL;
    g_last.line = 0;
    free(g_last.reason);
    g_last.reason = NULL;
}

void spt_Panic(const char *file, unsigned line, const char *expr) {
    fprintf(stderr, "%s:%u: assertion error: \"%s\"\n", file, line, expr);
    abort();
}

char *sptBytesString(uint64_t const bytes) {
    static const char *const suffix[] = {"B", "KB", "MB", "GB", "TB"};
    double size = (double)bytes;
    int k = 0;
    while (size > 1024 && k < 4) {
        size /= 1024.;
        ++k;
    }
    char *ret = NULL;
    if (asprintf(&ret, "%0.2f%s", size, suffix[k]) == -1) ret = NULL;
    return ret;
}

int sptgb_cuda_fail(cudaError_t e, const char *module, const char *file, unsigned line) {
    const int code = SPTERR_CUDA_ERROR + (int)e;
    spt_ComplainError(module, code, file, line, cudaGetErrorString(e));
    return code;
}

static void ctx_init_once(void) {
    const char *d = getenv("SPTGB_DEVICE");
    g_device = d ? atoi(d) : 0;
    cudaError_t e = cudaSetDevice(g_device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g_copy_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) g_init_err = sptgb_cuda_fail(e, "SpTns GPU init", __FILE__, __LINE__);
}

int sptgb_ctx(void) {
    pthread_once(&g_once, ctx_init_once);
    if (g_init_err) return g_init_err;
    /* The device is per host thread in the CUDA runtime. */
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != g_device) {
        cudaError_t e = cudaSetDevice(g_device);
        if (e != cudaSuccess) return sptgb_cuda_fail(e, "SpTns GPU init", __FILE__, __LINE__);
    }
    return 0;
}

/* Streaming multiprocessors of the library's device (grid caps of the
 * grid-stride kernels are multiples of it); looked up once. */
static _Atomic int g_sm_count = 0;

int sptgb_sm_count(void) {
    int n = atomic_load(&g_sm_count);
    if (n > 0) return n;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 1;   /* not cached: a later call retries */
    }
    atomic_store(&g_sm_count, n);
    return n;
}

cudaStream_t sptgb_stream(void) { return g_stream; }
cudaStream_t sptgb_copy_stream(void) { return g_copy_stream; }

void sptgb_count_launch(unsigned n) { atomic_fetch_add(&g_launches, (uint64_t)n); }
void sptgb_uncount_launch(uint64_t n) { atomic_fetch_sub(&g_launches, n); }

int sptgb_dbuf_reserve(sptgb_dbuf *b, size_t bytes) {
    if (bytes <= b->cap && b->ptr) return 0;
    if (b->ptr) {
        cudaFree(b->ptr);
        b->ptr = NULL;
        b->cap = 0;
    }
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&b->ptr, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b->ptr = NULL;
        return sptgb_cuda_fail(e, "SpTns GPU alloc", __FILE__, __LINE__);
    }
    b->cap = want;
    return 0;
}

void sptgb_dbuf_release(sptgb_dbuf *b) {
    if (b->ptr) cudaFree(b->ptr);
    b->ptr = NULL;
    b->cap = 0;
}

/* ------------------------------------------------------ public library -- */
const char *sptgbVersion(void) { return "sptgb 0.1 (sm_103a)"; }

int sptgbInit(int device) {
    if (device >= 0) {
        char buf[32];
        snprintf(buf, sizeof buf, "%d", device);
        setenv("SPTGB_DEVICE", buf, 0);
    }
    return sptgb_ctx();
}

void *sptgbStream(void) {
    if (sptgb_ctx()) return NULL;
    return (void *)g_stream;
}

uint64_t sptgbLaunchCount(void) { return atomic_load(&g_launches); }

/* SPTGB_SEED is read once, on the first use of the seed, whether or not a
 * device call came first; sptgbSetSeed overrides it. */
static pthread_once_t g_seed_once = PTHREAD_ONCE_INIT;
static void seed_from_env(void) {
    const char *s = getenv("SPTGB_SEED");
    if (s) g_seed = strtoull(s, NULL, 0);
}

void sptgbSetSeed(uint64_t seed) {
    pthread_once(&g_seed_once, seed_from_env);
    g_seed = seed;
}

uint64_t sptgb_seed_next(void) {
    /* Each randomised matrix gets its own stream of the seed. */
    static _Atomic uint64_t counter = 0;
    pthread_once(&g_seed_once, seed_from_env);
    return g_seed * 0x9E3779B97F4A7C15ULL + atomic_fetch_add(&counter, 1) + 1;
}

int sptCudaSetDevice(int device) { return sptgbInit(device); }

int sptCudaGetLastError(void) {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : SPTERR_CUDA_ERROR + (int)e;
}

/* ------------------------------------------------------------- timers -- */
struct sptTagTimer {
    int use_cuda;
    struct timespec start, stop;
    cudaEvent_t ev_start, ev_stop;
};

int sptNewTimer(sptTimer *timer, int use_cuda) {
    *timer = (sptTimer)calloc(1, sizeof(**timer));
    if (!*timer) return SPTERR_OS_ERROR;
    (*timer)->use_cuda = use_cuda;
    if (use_cuda) {
        SPTGB_CHECK(sptgb_ctx(), "Timer New");
        SPTGB_CUDA(cudaEventCreate(&(*timer)->ev_start), "Timer New");
        SPTGB_CUDA(cudaEventCreate(&(*timer)->ev_stop), "Timer New");
    }
    return 0;
}

int sptStartTimer(sptTimer timer) {
    if (timer->use_cuda) {
        SPTGB_CUDA(cudaEventRecord(timer->ev_start, g_stream), "Timer Start");
    } else {
        clock_gettime(CLOCK_MONOTONIC, &timer->start);
    }
    return 0;
}

int sptStopTimer(sptTimer timer) {
    if (timer->use_cuda) {
        SPTGB_CUDA(cudaEventRecord(timer->ev_stop, g_stream), "Timer Stop");
        SPTGB_CUDA(cudaEventSynchronize(timer->ev_stop), "Timer Stop");
    } else {
        clock_gettime(CLOCK_MONOTONIC, &timer->stop);
    }
    return 0;
}

double sptElapsedTime(const sptTimer timer) {
    if (timer->use_cuda) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, timer->ev_start, timer->ev_stop);
        return ms * 1e-3;
    }
    return (double)(timer->stop.tv_sec - timer->start.tv_sec) +
           (double)(timer->stop.tv_nsec - timer->start.tv_nsec) * 1e-9;
}

double sptPrintElapsedTime(const sptTimer timer, const char *name) {
    double t = sptElapsedTime(timer);
    printf("[%s]: %.9lf s\n", name, t);
    return t;
}

double sptPrintAverageElapsedTime(const sptTimer timer, const int niters, const char *name) {
    double t = sptElapsedTime(timer) / niters;
    printf("[%s]: %.9lf s\n", name, t);
    return t;
}

int sptFreeTimer(sptTimer timer) {
    if (timer->use_cuda) {
        cudaEventDestroy(timer->ev_start);
        cudaEventDestroy(timer->ev_stop);
    }
    free(timer);
    return 0;
}
