// lp_tune.cu — run-time tuning of a batch's split and launch shapes (lidar_gb300_batch.h).
//
// A tuning fixes how a batch is split into concurrent parts (how many, which scans go to each)
// and the launch shapes of the grid-strided and persistent kernels: the hull kernel's CTA/warp
// boundary by cluster size, its CTAs per SM, and the CTAs per SM of the polar-cell sort and the
// vote-weight pass. Results never depend on it (every path is exact); only the step time does.
// Tunings are kept per bucket of a batch (scan count class, and the ring-count and azimuth-width
// classes holding most points) in a host table; lp_autotune fills it by timing candidates on the
// scans given, as prepared batches replayed from CUDA graphs. No counterpart in the reference.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <utility>
#include <vector>

#include "lp_runtime.hpp"

struct lp_tuning_table
{
    std::map<uint32_t, std::pair<lp_tuning_key, std::pair<lp_tuning, float>>> entries;
};

namespace lprt
{
lp_status create_batch(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans, uint32_t nscans,
                       const lp_tuning& tune, lp_batch** out);

lp_tuning tuning_default()
{
    lp_tuning t;
    t.parts = 0;
    t.balance_parts = 0;
    t.hull_cta_min = 512;
    t.hull_ctas_per_sm = 2;
    t.cell_ctas_per_sm = 8;
    t.jcp_ctas_per_sm = 8;
    return t;
}

uint32_t key_index(const lp_tuning_key& k)
{
    return (k.scans_class * 3u + k.ring_class) * 3u + k.azimuth_class;
}

lp_tuning_key key_of(const lp_scan_input* scans, uint32_t nscans)
{
    lp_tuning_key k{};
    k.scans_class = nscans <= 1u ? 0u : (nscans < 16u ? 1u : (nscans < 32u ? 2u : (nscans < 64u ? 3u : 4u)));
    uint64_t ring_pts[3] = {0, 0, 0}, az_pts[3] = {0, 0, 0};
    for (uint32_t i = 0; i < nscans; ++i)
    {
        const int32_t H = scans[i].seg.image_height, W = scans[i].seg.image_width;
        const uint64_t n = scans[i].n;
        ring_pts[H <= 32 ? 0 : (H <= 64 ? 1 : 2)] += n;
        az_pts[W <= 1024 ? 0 : (W <= 2048 ? 1 : 2)] += n;
    }
    for (uint32_t c = 1; c < 3; ++c)
    {
        if (ring_pts[c] > ring_pts[k.ring_class])
            k.ring_class = c;
        if (az_pts[c] > az_pts[k.azimuth_class])
            k.azimuth_class = c;
    }
    return k;
}

lp_tuning tuning_for(const lp_context* ctx, const lp_scan_input* scans, uint32_t nscans)
{
    if (ctx && !ctx->tuning.empty() && (scans || nscans == 0))
    {
        const auto it = ctx->tuning.find(key_index(key_of(scans, nscans)));
        if (it != ctx->tuning.end())
            return it->second;
    }
    return tuning_default();
}

uint32_t part_count(const lp_tuning& t, uint32_t nscans)
{
    if (nscans <= 1u)
        return 1u;
    if (t.parts == 0u)
        return nscans < 16u ? 1u : std::min(8u, nscans / 8u);
    return std::min(t.parts, nscans);
}

std::vector<std::vector<uint32_t>> assign_parts(const lp_scan_input* scans, uint32_t nscans, uint32_t parts,
                                                bool balance)
{
    std::vector<std::vector<uint32_t>> where(parts);
    if (!balance)
    {
        for (uint32_t i = 0; i < nscans; ++i)
            where[i % parts].push_back(i);
        return where;
    }
    // largest scan first to the part holding the fewest points (the lowest part on ties); each
    // part keeps its scans in batch order
    std::vector<uint32_t> order(nscans);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return scans[a].n > scans[b].n; });
    std::vector<uint64_t> load(parts, 0);
    for (const uint32_t i : order)
    {
        uint32_t best = 0;
        for (uint32_t k = 1; k < parts; ++k)
            if (load[k] < load[best])
                best = k;
        load[best] += scans[i].n;
        where[best].push_back(i);
    }
    for (auto& w : where)
        std::sort(w.begin(), w.end());
    return where;
}
} // namespace lprt

extern "C" {

void lp_tuning_default(lp_tuning* t)
{
    if (t)
        *t = lprt::tuning_default();
}

lp_status lp_tuning_validate(const lp_tuning* t)
{
    if (!t)
        return LP_ERR_BAD_ARG;
    const bool ok = t->parts <= 8u && t->balance_parts <= 1u && t->hull_cta_min >= 64u && t->hull_cta_min <= 512u &&
                    t->hull_ctas_per_sm >= 1u && t->hull_ctas_per_sm <= 4u && t->cell_ctas_per_sm >= 1u &&
                    t->cell_ctas_per_sm <= 16u && t->jcp_ctas_per_sm >= 1u && t->jcp_ctas_per_sm <= 16u;
    return ok ? LP_OK : LP_ERR_BAD_ARG;
}

lp_status lp_tuning_key_of(const lp_scan_input* scans, uint32_t nscans, lp_tuning_key* out)
{
    if (!out || (!scans && nscans))
        return LP_ERR_BAD_ARG;
    *out = lprt::key_of(scans, nscans);
    return LP_OK;
}

lp_status lp_tuning_table_create(lp_tuning_table** out)
{
    if (!out)
        return LP_ERR_BAD_ARG;
    *out = new lp_tuning_table();
    return LP_OK;
}

void lp_tuning_table_destroy(lp_tuning_table* table)
{
    delete table;
}

static bool key_ok(const lp_tuning_key* k)
{
    return k && k->scans_class <= 4u && k->ring_class <= 2u && k->azimuth_class <= 2u;
}

lp_status lp_tuning_table_set(lp_tuning_table* table, const lp_tuning_key* key, const lp_tuning* tuning, float ms)
{
    if (!table || !key_ok(key) || lp_tuning_validate(tuning) != LP_OK)
        return LP_ERR_BAD_ARG;
    table->entries[lprt::key_index(*key)] = {*key, {*tuning, ms}};
    return LP_OK;
}

int32_t lp_tuning_table_get(const lp_tuning_table* table, const lp_tuning_key* key, lp_tuning* out, float* ms)
{
    if (out)
        *out = lprt::tuning_default();
    if (ms)
        *ms = 0.0F;
    if (!table || !key_ok(key))
        return 0;
    const auto it = table->entries.find(lprt::key_index(*key));
    if (it == table->entries.end())
        return 0;
    if (out)
        *out = it->second.second.first;
    if (ms)
        *ms = it->second.second.second;
    return 1;
}

uint32_t lp_tuning_table_size(const lp_tuning_table* table)
{
    return table ? static_cast<uint32_t>(table->entries.size()) : 0u;
}

lp_status lp_tuning_table_save(const lp_tuning_table* table, const char* path)
{
    if (!table || !path)
        return LP_ERR_BAD_ARG;
    FILE* f = std::fopen(path, "w");
    if (!f)
        return LP_ERR_BAD_ARG;
    std::fprintf(f, "# lp_tuning 1: scans_class ring_class azimuth_class parts balance_parts hull_cta_min "
                    "hull_ctas_per_sm cell_ctas_per_sm jcp_ctas_per_sm ms\n");
    for (const auto& e : table->entries)
    {
        const lp_tuning_key& k = e.second.first;
        const lp_tuning& t = e.second.second.first;
        std::fprintf(f, "%u %u %u %u %u %u %u %u %u %.6g\n", k.scans_class, k.ring_class, k.azimuth_class, t.parts,
                     t.balance_parts, t.hull_cta_min, t.hull_ctas_per_sm, t.cell_ctas_per_sm, t.jcp_ctas_per_sm,
                     static_cast<double>(e.second.second.second));
    }
    const bool ok = std::fclose(f) == 0;
    return ok ? LP_OK : LP_ERR_BAD_ARG;
}

lp_status lp_tuning_table_load(lp_tuning_table* table, const char* path)
{
    if (!table || !path)
        return LP_ERR_BAD_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f)
        return LP_ERR_BAD_ARG;
    char line[512];
    lp_status st = LP_OK;
    std::vector<std::pair<lp_tuning_key, std::pair<lp_tuning, float>>> got;
    while (st == LP_OK && std::fgets(line, sizeof(line), f))
    {
        const char* p = line;
        while (*p == ' ' || *p == '\t')
            ++p;
        if (*p == '#' || *p == '\n' || *p == '\r' || *p == '\0')
            continue;
        lp_tuning_key k{};
        lp_tuning t{};
        float ms = 0.0F;
        const int n = std::sscanf(p, "%u %u %u %u %u %u %u %u %u %f", &k.scans_class, &k.ring_class, &k.azimuth_class,
                                  &t.parts, &t.balance_parts, &t.hull_cta_min, &t.hull_ctas_per_sm, &t.cell_ctas_per_sm,
                                  &t.jcp_ctas_per_sm, &ms);
        if (n != 10 || !key_ok(&k) || lp_tuning_validate(&t) != LP_OK)
            st = LP_ERR_BAD_ARG;
        else
            got.push_back({k, {t, ms}});
    }
    std::fclose(f);
    if (st != LP_OK)
        return st; // a malformed file changes nothing
    for (const auto& e : got)
        table->entries[lprt::key_index(e.first)] = {e.first, e.second};
    return LP_OK;
}

lp_status lp_context_set_tuning_table(lp_context* ctx, const lp_tuning_table* table)
{
    if (!ctx)
        return LP_ERR_BAD_ARG;
    ctx->tuning.clear();
    if (table)
        for (const auto& e : table->entries)
            ctx->tuning[e.first] = e.second.second.first;
    return LP_OK;
}

lp_status lp_autotune(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans, uint32_t nscans,
                      uint32_t iters, lp_tuning_table* table, lp_tuning* best, lp_autotune_report* report,
                      float* trial_ms, lp_tuning* trial_cfg, uint32_t trial_cap)
{
    if (!ctx || !cfg || !scans || nscans == 0 || iters == 0)
        return lprt::fail(ctx, LP_ERR_BAD_ARG, "lp_autotune: null argument, no scans or no iterations");
    const lp_tuning_key key = lprt::key_of(scans, nscans);
    lp_tuning cur = lprt::tuning_default();
    if (table)
        lp_tuning_table_get(table, &key, &cur, nullptr);
    uint32_t trials = 0;
    // one candidate: a prepared batch with this tuning, one warm-up execution, then `iters` timed
    // back to back (no L2 flush between them: executions follow one another as in a stream of
    // batches, and as the batch's throughput is measured)
    auto time_it = [&](const lp_tuning& t, float& ms) -> lp_status {
        lp_batch* B = nullptr;
        lp_status st = lprt::create_batch(ctx, cfg, scans, nscans, t, &B);
        if (st != LP_OK)
            return st;
        st = lp_batch_capture_graph(ctx, B);
        if (st == LP_OK)
            st = lp_batch_execute(ctx, B);
        if (st == LP_OK)
            st = lp_context_synchronize(ctx);
        if (st == LP_OK)
            st = lp_batch_time(ctx, B, iters, 0, &ms);
        lp_batch_destroy(ctx, B);
        if (st == LP_OK)
        {
            if (trial_ms && trials < trial_cap)
                trial_ms[trials] = ms;
            if (trial_cfg && trials < trial_cap)
                trial_cfg[trials] = t;
            ++trials;
        }
        return st;
    };
    float cur_ms = 0.0F;
    const lp_status st0 = time_it(cur, cur_ms);
    if (st0 != LP_OK)
        return st0;
    const float start_ms = cur_ms;
    // coordinate descent: each field in turn over its candidates, keeping a change only when it
    // is at least 1 % faster than the current choice
    struct Field
    {
        uint32_t lp_tuning::*member;
        std::vector<uint32_t> values;
    };
    const std::vector<Field> fields = {
        {&lp_tuning::parts, {0u, 1u, 2u, 4u, 8u}},
        {&lp_tuning::balance_parts, {0u, 1u}},
        {&lp_tuning::hull_cta_min, {128u, 256u, 512u}},
        {&lp_tuning::hull_ctas_per_sm, {1u, 2u, 3u, 4u}},
        {&lp_tuning::cell_ctas_per_sm, {4u, 8u, 12u}},
        {&lp_tuning::jcp_ctas_per_sm, {4u, 8u, 12u}},
    };
    for (const Field& f : fields)
    {
        for (const uint32_t v : f.values)
        {
            lp_tuning t = cur;
            t.*(f.member) = v;
            if (v == cur.*(f.member))
                continue;
            // candidates that give the same batch as the current choice are not timed again
            if (f.member == &lp_tuning::parts && lprt::part_count(t, nscans) == lprt::part_count(cur, nscans))
                continue;
            if (f.member == &lp_tuning::balance_parts && lprt::part_count(cur, nscans) == 1u)
                continue;
            float ms = 0.0F;
            const lp_status st = time_it(t, ms);
            if (st != LP_OK)
                return st;
            if (ms < 0.99F * cur_ms)
            {
                cur = t;
                cur_ms = ms;
            }
        }
    }
    if (table && lp_tuning_table_set(table, &key, &cur, cur_ms) != LP_OK)
        return LP_ERR_INTERNAL;
    if (best)
        *best = cur;
    if (report)
    {
        report->trials = trials;
        report->start_ms = start_ms;
        report->best_ms = cur_ms;
    }
    return LP_OK;
}

} // extern "C"
