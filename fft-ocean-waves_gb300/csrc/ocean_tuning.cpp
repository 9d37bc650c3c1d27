// ocean_tuning.cpp -- the per-N launch configuration (ocean_get_tuning /
// ocean_set_tuning of include/ocean.h).  The defaults are the compiled-in
// table tuning_table.inc, which tune.py writes from GB300 measurements; a
// process may replace an entry at run time (the tuner does, to measure the
// candidates).  No counterpart in the reference, which has one fixed dispatch
// shape per shader.
#include <atomic>
#include <string>

#include "ocean.h"
#include "ocean_host.h"
#include "ocean_internal.h"

namespace {

struct Entry {
    int N, row_overlap, row_ctas_per_sm, wave_mib, col_fused, row_variant;
};
constexpr Entry kTable[] = {
#include "tuning_table.inc"
};
constexpr int kSizes = (int)(sizeof(kTable) / sizeof(kTable[0]));
static_assert(kSizes == 7, "one entry per supported N (32 .. 2048)");

struct Live {
    std::atomic<int> row_overlap, row_ctas_per_sm, wave_mib, col_fused, row_variant;
};

// The live table, filled from kTable on first use (thread-safe static
// initialisation).
Live* live()
{
    static Live* table = [] {
        static Live l[kSizes];
        for (int i = 0; i < kSizes; ++i) {
            l[i].row_overlap.store(kTable[i].row_overlap);
            l[i].row_ctas_per_sm.store(kTable[i].row_ctas_per_sm);
            l[i].wave_mib.store(kTable[i].wave_mib);
            l[i].col_fused.store(kTable[i].col_fused);
            l[i].row_variant.store(kTable[i].row_variant);
        }
        return l;
    }();
    return table;
}

// The row-pass variants that exist for size N: below 512 only the every-warp
// pass (1); variants 3, 4 and 5 (32 x 32 lines) at N = 1024 only, elsewhere
// they read as the same pass with the default lines (0, 1 and 0).
int row_variant_for(int N, int v)
{
    if (N < 512) return 1;
    if ((v == 3 || v == 5) && N != 1024) return 0;
    if (v == 4 && N != 1024) return 1;
    return v;
}

int slot(int N)
{
    for (int i = 0; i < kSizes; ++i)
        if (kTable[i].N == N) return i;
    return -1;
}

}  // namespace

namespace ocean {

Tuning tuning_for(int N)
{
    const int i = slot(N);
    if (i < 0) return Tuning{0, 0, 64, 0, 1};
    const Live& l = live()[i];
    return Tuning{l.row_overlap.load(std::memory_order_relaxed), l.row_ctas_per_sm.load(std::memory_order_relaxed),
                  l.wave_mib.load(std::memory_order_relaxed),
                  ocean::col_fused_available(N) ? l.col_fused.load(std::memory_order_relaxed) : 0,
                  row_variant_for(N, l.row_variant.load(std::memory_order_relaxed))};
}

}  // namespace ocean

using namespace ocean::host;

extern "C" int ocean_get_tuning(int32_t N, ocean_tuning* out)
{
    if (!out) return fail(OCEAN_ERR_INVALID, "out is NULL");
    if (slot(N) < 0) return fail(OCEAN_ERR_INVALID, "no tuning entry for N = " + std::to_string(N));
    const ocean::Tuning t = ocean::tuning_for(N);
    out->row_overlap      = t.row_overlap;
    out->row_ctas_per_sm  = t.row_ctas_per_sm;
    out->wave_mib         = t.wave_mib;
    out->col_fused        = t.col_fused;
    out->row_variant      = t.row_variant;
    return OCEAN_OK;
}

extern "C" int ocean_set_tuning(int32_t N, const ocean_tuning* cfg)
{
    if (!cfg) return fail(OCEAN_ERR_INVALID, "cfg is NULL");
    const int i = slot(N);
    if (i < 0) return fail(OCEAN_ERR_INVALID, "no tuning entry for N = " + std::to_string(N));
    if ((cfg->row_overlap != 0 && cfg->row_overlap != 1) || cfg->row_ctas_per_sm < 0 || cfg->row_ctas_per_sm > 32 ||
        cfg->wave_mib < 1 || cfg->wave_mib > 4096 || (cfg->col_fused != 0 && cfg->col_fused != 2 && cfg->col_fused != 4) ||
        cfg->row_variant < 0 || cfg->row_variant > 5)
        return fail(OCEAN_ERR_INVALID, "tuning values out of range");
    Live& l = live()[i];
    l.row_overlap.store(cfg->row_overlap);
    l.row_ctas_per_sm.store(cfg->row_ctas_per_sm);
    l.wave_mib.store(cfg->wave_mib);
    l.col_fused.store(cfg->col_fused);
    l.row_variant.store(cfg->row_variant);
    return OCEAN_OK;
}
