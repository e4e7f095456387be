// common.cu -- context, error reporting and budgeted device allocation.
#include "internal.h"

#include <cstdarg>
#include <mutex>
#include <unordered_map>
#include <vector>

namespace amie {

std::atomic<uint64_t> g_launches{0};

static thread_local std::string t_error;

void set_error(const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_error = buf;
}

amie_status dev_alloc(Ctx *ctx, void **p, size_t bytes)
{
    *p = nullptr;
    if (ctx->budget && ctx->allocated.load() + bytes > ctx->budget) {
        set_error("HBM budget exceeded: %llu + %llu > %llu bytes", (unsigned long long)ctx->allocated.load(),
                  (unsigned long long)bytes, (unsigned long long)ctx->budget);
        return AMIE_OOM;
    }
    cudaError_t e = ctx->pool ? cudaMallocFromPoolAsync(p, bytes, ctx->pool, ctx->stream) : cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        set_error("cudaMalloc(%llu): %s", (unsigned long long)bytes, cudaGetErrorString(e));
        cudaGetLastError();
        *p = nullptr;
        return AMIE_OOM;
    }
    ctx->allocated += bytes;
    return AMIE_OK;
}

static thread_local cudaStream_t t_free_stream = nullptr;

void set_free_stream(cudaStream_t st) { t_free_stream = st; }

void dev_free(Ctx *ctx, void *p, size_t bytes)
{
    if (!p) return;
    if (ctx && ctx->pool) cudaFreeAsync(p, t_free_stream ? t_free_stream : ctx->stream);
    else cudaFree(p);
    if (ctx) ctx->allocated -= bytes;
}

static std::mutex g_pinned_mu;
static std::unordered_map<size_t, std::vector<void *>> g_pinned_free;

void *pinned_get(size_t bytes)
{
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        auto &v = g_pinned_free[bytes];
        if (!v.empty()) {
            void *p = v.back();
            v.pop_back();
            return p;
        }
    }
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void pinned_put(void *p, size_t bytes)
{
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    g_pinned_free[bytes].push_back(p);
}

}  // namespace amie

using namespace amie;

extern "C" const char *amie_last_error(void) { return t_error.c_str(); }

extern "C" int32_t amie_abi_version(void) { return AMIE_GPU_ABI_VERSION; }

extern "C" uint64_t amie_kernel_launches(void) { return g_launches.load(); }

extern "C" amie_status amie_ctx_create(const amie_config *cfg, amie_ctx **out)
{
    if (!out) return AMIE_BAD_INPUT;
    *out = nullptr;
    int dev = cfg ? cfg->device : 0;
    int count = 0;
    AMIE_CUDA(cudaGetDeviceCount(&count));
    if (dev < 0 || dev >= count) {
        set_error("device %d not present (%d devices)", dev, count);
        return AMIE_BAD_INPUT;
    }
    AMIE_CUDA(cudaSetDevice(dev));
    amie_ctx *c = new amie_ctx();
    c->device = dev;
    c->budget = cfg ? cfg->hbm_budget_bytes : 0;
    c->verbose = cfg ? cfg->verbose : 0;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) c->num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
        cudaMallocHost((void **)&c->h_scalars, 64 * sizeof(double)) != cudaSuccess) {
        set_error("stream/event/pinned allocation failed");
        delete c;
        return AMIE_CUDA_ERROR;
    }
    *out = c;
    return AMIE_OK;
}

extern "C" amie_status amie_ctx_destroy(amie_ctx *ctx)
{
    if (!ctx) return AMIE_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->h_scalars) cudaFreeHost(ctx->h_scalars);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return AMIE_OK;
}
