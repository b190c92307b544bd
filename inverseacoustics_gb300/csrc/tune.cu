// Kernel-variant autotuner (see tune.h).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <map>
#include <mutex>
#include "tune.h"

namespace ia {

namespace {

struct KeyLess {
    bool operator()(const TuneKey &a, const TuneKey &b) const
    {
        if (a.kernel != b.kernel) return a.kernel < b.kernel;
        if (a.device != b.device) return a.device < b.device;
        return memcmp(a.v, b.v, sizeof(a.v)) < 0;
    }
};

std::mutex g_mu;
std::map<TuneKey, int, KeyLess> g_table;
int g_enabled = -1;   // -1: not read yet
bool g_file_read = false;

const char *tune_file() { return getenv("IA_TUNE_FILE"); }

void read_file_locked()
{
    g_file_read = true;
    const char *fn = tune_file();
    if (!fn || !*fn) return;
    FILE *fp = fopen(fn, "r");
    if (!fp) return;
    TuneKey k;
    int var;
    while (fscanf(fp, "%d %d %d %d %d %d %d %d %d %d %d", &k.kernel, &k.device, &k.v[0], &k.v[1], &k.v[2], &k.v[3],
                  &k.v[4], &k.v[5], &k.v[6], &k.v[7], &var) == 11)
        g_table[k] = var;
    fclose(fp);
}

void append_file(const TuneKey &k, int var)
{
    const char *fn = tune_file();
    if (!fn || !*fn) return;
    FILE *fp = fopen(fn, "a");
    if (!fp) return;
    fprintf(fp, "%d %d %d %d %d %d %d %d %d %d %d\n", k.kernel, k.device, k.v[0], k.v[1], k.v[2], k.v[3], k.v[4],
            k.v[5], k.v[6], k.v[7], var);
    fclose(fp);
}

bool enabled_locked()
{
    if (g_enabled < 0) {
        const char *e = getenv("IA_TUNE");
        g_enabled = (e && e[0] == '0') ? 0 : 1;
    }
    return g_enabled == 1;
}

}  // namespace

int TuneScratch::init(const void *src, size_t bytes)
{
    IA_CUDA_TRY(cudaMallocAsync(&p, bytes, ctx->stream));
    IA_CUDA_TRY(cudaMemcpyAsync(p, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return IA_OK;
}

TuneScratch::~TuneScratch()
{
    if (p) cudaFreeAsync(p, ctx->stream);
}

int tune_select(ia_context *ctx, TuneKey key, int nvar, const std::function<int(int)> &run)
{
    key.device = ctx->device;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_file_read) read_file_locked();
        auto it = g_table.find(key);
        if (it != g_table.end() && it->second < nvar) return it->second;
        if (!enabled_locked() || ctx->capturing || ctx->no_tune || nvar < 2) return 0;
    }
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return 0;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return 0;
    }
    int best = 0;
    float best_ms = 1e30f;
    bool ok = true;
    for (int v = 0; v < nvar && ok; ++v) {
        if (run(v) != IA_OK) { ok = false; break; }           // warm-up (and instruction cache)
        cudaEventRecord(e0, ctx->stream);
        for (int r = 0; r < 3 && ok; ++r) ok = run(v) == IA_OK;
        cudaEventRecord(e1, ctx->stream);
        if (!ok || cudaEventSynchronize(e1) != cudaSuccess) { ok = false; break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) { best_ms = ms; best = v; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!ok) return 0;
    std::lock_guard<std::mutex> lk(g_mu);
    g_table[key] = best;
    append_file(key, best);
    return best;
}

}  // namespace ia

extern "C" {

// number of tuned entries in the process-wide table
int ia_tune_table_size(void)
{
    std::lock_guard<std::mutex> lk(ia::g_mu);
    return (int)ia::g_table.size();
}

// forget all tuned choices (the next calls tune again); also re-reads IA_TUNE
void ia_tune_reset(void)
{
    std::lock_guard<std::mutex> lk(ia::g_mu);
    ia::g_table.clear();
    ia::g_enabled = -1;
    ia::g_file_read = false;
}

}  // extern "C"
