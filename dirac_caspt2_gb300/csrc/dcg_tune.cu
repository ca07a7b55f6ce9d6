// The autotuner's table (see dcg_common.cuh): tuned choices per decision and problem shape,
// shared by every context of the process, and its C ABI.
#include <cstdio>
#include <mutex>
#include <vector>

#include "dcg_common.cuh"

namespace dcg {

namespace {

struct TuneEntry {
    int choice, ncand;
    float best_ms, heuristic_ms;
};

std::mutex g_mu;
std::map<TuneKey, TuneEntry> g_table;
int g_mode = -1;   // -1: not read yet
bool g_loaded = false;

int mode_locked() {
    if (g_mode < 0) {
        const char *e = getenv("DCG_AUTOTUNE");
        g_mode = (e && e[0] == '0') ? 0 : 1;
    }
    return g_mode;
}

// With DCG_TUNE_FILE set, the table persists in that text file, one entry per line
// ("kind ops m n k flags choice ncand best_ms heuristic_ms"): entries are read at the first
// lookup and every new entry is appended, so another process (a profiler's run of the same
// workload, a service restart) reuses the choices without trials.
const char *tune_file() { return getenv("DCG_TUNE_FILE"); }

void load_locked() {
    if (g_loaded) return;
    g_loaded = true;
    const char *f = tune_file();
    if (!f || !f[0]) return;
    FILE *fp = fopen(f, "r");
    if (!fp) return;
    TuneKey k;
    TuneEntry e;
    while (fscanf(fp, "%d %d %d %d %d %d %d %d %f %f", &k.kind, &k.ops, &k.m, &k.n, &k.k, &k.flags, &e.choice,
                  &e.ncand, &e.best_ms, &e.heuristic_ms) == 10)
        if (e.choice >= 0 && e.choice < e.ncand) g_table.emplace(k, e);
    fclose(fp);
}

void save_locked(const TuneKey &k, const TuneEntry &e) {
    const char *f = tune_file();
    if (!f || !f[0]) return;
    FILE *fp = fopen(f, "a");
    if (!fp) return;
    fprintf(fp, "%d %d %d %d %d %d %d %d %.6f %.6f\n", k.kind, k.ops, k.m, k.n, k.k, k.flags, e.choice, e.ncand,
            e.best_ms, e.heuristic_ms);
    fclose(fp);
}

}  // namespace

int autotune_run(Context &c, const TuneKey &key, int ncand, bool trial_ok, void (*fn)(void *, int), void *arg) {
    {
        std::lock_guard<std::mutex> lk(g_mu);
        load_locked();
        auto it = g_table.find(key);
        if (it != g_table.end()) return it->second.choice < ncand ? it->second.choice : 0;
        if (mode_locked() == 0 || ncand < 2 || !trial_ok || !c.tune_trials) return 0;
    }
    // untimed pass: every candidate once (workspace growth, first-launch costs)
    for (int q = 0; q < ncand; q++) fn(arg, q);
    cudaEvent_t a, b;
    DCG_CUDA(cudaEventCreate(&a));
    DCG_CUDA(cudaEventCreate(&b));
    std::vector<float> best(ncand, 1e30f);
    for (int rep = 0; rep < 2; rep++)
        for (int q = 0; q < ncand; q++) {
            DCG_CUDA(cudaEventRecord(a, c.stream));
            fn(arg, q);
            DCG_CUDA(cudaEventRecord(b, c.stream));
            DCG_CUDA(cudaEventSynchronize(b));
            float ms = 0.f;
            DCG_CUDA(cudaEventElapsedTime(&ms, a, b));
            best[q] = std::min(best[q], ms);
        }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    int pick = 0;
    for (int q = 1; q < ncand; q++)
        if (best[q] < best[pick]) pick = q;
    std::lock_guard<std::mutex> lk(g_mu);
    auto ins = g_table.emplace(key, TuneEntry{pick, ncand, best[pick], best[0]});
    if (ins.second) save_locked(key, ins.first->second);
    return ins.first->second.choice;   // a concurrent tuner of the same key may have won
}

}  // namespace dcg

extern "C" {

int dcg_autotune_mode(int32_t mode) {
    std::lock_guard<std::mutex> lk(dcg::g_mu);
    const int prev = dcg::mode_locked();
    if (mode == 0 || mode == 1) dcg::g_mode = mode;
    else if (mode == 2) dcg::g_table.clear();
    return prev;
}

int32_t dcg_autotune_entries(dcg_tune_entry *out, int32_t max_entries) {
    std::lock_guard<std::mutex> lk(dcg::g_mu);
    dcg::load_locked();
    int32_t n = 0;
    for (const auto &kv : dcg::g_table) {
        if (out && n < max_entries) {
            dcg_tune_entry &e = out[n];
            e.kind = kv.first.kind;
            e.ops = kv.first.ops;
            e.m = kv.first.m;
            e.n = kv.first.n;
            e.k = kv.first.k;
            e.flags = kv.first.flags;
            e.choice = kv.second.choice;
            e.ncand = kv.second.ncand;
            e.best_ms = kv.second.best_ms;
            e.heuristic_ms = kv.second.heuristic_ms;
        }
        n++;
    }
    return n;
}

}  // extern "C"
