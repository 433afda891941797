// Autotuner of the batched Poisson solve: searches the tunables of a size
// mix (inner cycles, the size below which levels run in one block, sweeps
// fused per tile pass, execution mode and optionally the smoothing sweeps)
// by timing real solves of the caller's right-hand side on the device, and
// remembers the winner per (device, size mix, precision, tolerance) in
// memory and in an optional text cache file.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gbcommon.cuh"

namespace {

std::mutex g_tune_mu;
std::map<std::string, gb_batch_tuning> g_tune_mem;

// The cache key: device, precision, smoothing, tolerance and the multiset
// of sizes (the order of the problems does not matter to the tunables).
std::string tune_key(int nprob, const int *n, int precision, int nu1, int nu2, int tune_nu, double rtol,
                     int max_cycles)
{
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    memset(&prop, 0, sizeof(prop));
    cudaGetDeviceProperties(&prop, dev);
    std::map<int, int> count;
    for (int p = 0; p < nprob; ++p) count[n[p]]++;
    std::string k = "v1|";
    for (const char *c = prop.name; *c; ++c) k += (*c == ' ' || *c == '|') ? '_' : *c;
    char buf[256];
    snprintf(buf, sizeof(buf), "|sm%d|p%d|nu%d,%d,%d|rtol%.6e|mc%d|", prop.multiProcessorCount, precision, nu1, nu2,
             tune_nu, rtol, max_cycles);
    k += buf;
    for (const auto &kv : count) {
        snprintf(buf, sizeof(buf), "%dx%d,", kv.first, kv.second);
        k += buf;
    }
    return k;
}

bool cache_lookup(const char *path, const std::string &key, gb_batch_tuning *t)
{
    if (!path) return false;
    FILE *fp = fopen(path, "r");
    if (!fp) return false;
    char line[8192];
    bool found = false;
    while (fgets(line, sizeof(line), fp)) {
        char *sep = strstr(line, " => ");
        if (!sep) continue;
        *sep = 0;
        if (key != line) continue;
        gb_batch_tuning c;
        memset(&c, 0, sizeof(c));
        if (sscanf(sep + 4, "nu1=%d nu2=%d inner=%d local_n=%d fuse=%d exec=%d ms=%lf", &c.nu1, &c.nu2, &c.inner,
                   &c.local_n, &c.fuse, &c.exec, &c.ms) == 7) {
            *t = c;   // the last matching line wins
            found = true;
        }
    }
    fclose(fp);
    return found;
}

void cache_store(const char *path, const std::string &key, const gb_batch_tuning &t)
{
    if (!path) return;
    FILE *fp = fopen(path, "a");
    if (!fp) return;   // the cache is advisory
    fprintf(fp, "%s => nu1=%d nu2=%d inner=%d local_n=%d fuse=%d exec=%d ms=%.6f\n", key.c_str(), t.nu1, t.nu2,
            t.inner, t.local_n, t.fuse, t.exec, t.ms);
    fclose(fp);
}

}  // namespace

extern "C" int gb_batch_autotune(int nprob, const int *n, int precision, int nu1, int nu2, int tune_nu, double rtol,
                                 int max_cycles, const double *d_f, double *d_psi, int reps, const char *cache_path,
                                 gb_batch_tuning *best, gb_batch_tuning *table, int table_cap, int *table_len,
                                 int *from_cache)
{
    if (table_len) *table_len = 0;
    if (from_cache) *from_cache = 0;
    if (!best || !n || nprob <= 0 || !d_f || !d_psi || reps < 1 || (table_cap > 0 && !table) ||
        (precision != GB_BATCH_FP64 && precision != GB_BATCH_MIXED && precision != GB_BATCH_MIXED_F64OUTER)) {
        gb_set_error("gb_batch_autotune: invalid argument");
        return GB_ERR_INVALID;
    }
    if (!cache_path) cache_path = getenv("GB300_BATCH_TUNE_CACHE");
    const std::string key = tune_key(nprob, n, precision, nu1, nu2, tune_nu, rtol, max_cycles);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_mem.find(key);
        if (it != g_tune_mem.end()) {
            *best = it->second;
            if (from_cache) *from_cache = 1;
            return GB_OK;
        }
        gb_batch_tuning c;
        if (cache_lookup(cache_path, key, &c)) {
            g_tune_mem[key] = c;
            *best = c;
            if (from_cache) *from_cache = 1;
            return GB_OK;
        }
    }
    // candidates
    std::vector<std::pair<int, int>> nus{{nu1, nu2}};
    if (tune_nu) {
        const int extra[5][2] = {{1, 1}, {1, 2}, {2, 1}, {2, 2}, {3, 3}};
        for (auto &e : extra)
            if (std::find(nus.begin(), nus.end(), std::make_pair(e[0], e[1])) == nus.end()) nus.push_back({e[0], e[1]});
    }
    const bool fp64 = precision == GB_BATCH_FP64;
    std::vector<int> inners = fp64 ? std::vector<int>{1} : std::vector<int>{2, 3, 4, 5};
    std::vector<int> locals = fp64 ? std::vector<int>{33, 65} : std::vector<int>{33, 65, 129};
    std::vector<gb_batch_tuning> cands;
    for (auto &nu : nus)
        for (int in : inners)
            for (int ln : locals)
                for (int fu = 1; fu <= 2; ++fu)
                    for (int ex = 0; ex <= 1; ++ex) {
                        gb_batch_tuning t;
                        memset(&t, 0, sizeof(t));
                        t.nu1 = nu.first;
                        t.nu2 = nu.second;
                        t.inner = in;
                        t.local_n = ln;
                        t.fuse = fu;
                        t.exec = ex;
                        cands.push_back(t);
                    }
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    GB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaError_t ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaStreamDestroy(s);
        gb_set_error("gb_batch_autotune: events: %s", cudaGetErrorString(ce));
        return GB_ERR_CUDA;
    }
    int ntab = 0, nok = 0;
    gb_batch_tuning win;
    memset(&win, 0, sizeof(win));
    win.ms = -1.0;
    int rc = GB_OK;
    for (gb_batch_tuning &t : cands) {
        gb_batch *b = nullptr;
        int st = gb_batch_create_tuned(nprob, n, precision, rtol, max_cycles, &t, &b);
        if (st == GB_ERR_ALLOC || st == GB_ERR_CUDA) { rc = st; break; }
        if (st != GB_OK) continue;   // not available here (e.g. no cooperative launch)
        st = gb_batch_solve_device(b, d_f, d_psi, nullptr, nullptr, s);
        float ms = 0.f;
        if (st == GB_OK) {
            cudaEventRecord(e0, s);
            for (int r = 0; r < reps && st == GB_OK; ++r) st = gb_batch_solve_device(b, d_f, d_psi, nullptr, nullptr, s);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
        }
        gb_batch_destroy(b);
        if (st == GB_ERR_CUDA) { rc = st; break; }
        if (st != GB_OK) continue;   // did not converge within max_cycles, or timed out
        t.ms = ms / reps;
        ++nok;
        if (table && ntab < table_cap) table[ntab++] = t;
        if (win.ms < 0.0 || t.ms < win.ms) win = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    if (table_len) *table_len = ntab;
    if (rc != GB_OK) return rc;
    if (nok == 0) {
        gb_set_error("gb_batch_autotune: no candidate solved the batch to the tolerance");
        return GB_MAXSWEEPS;
    }
    *best = win;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_mem[key] = win;
    cache_store(cache_path, key, win);
    return GB_OK;
}
