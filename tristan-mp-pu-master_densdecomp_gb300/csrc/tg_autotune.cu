// Autotuner: picks the tile shape (and with it the particles per tile) and
// the re-sort cadence for a given domain and plasma by timing short runs of
// the fused lap on the device. Candidates that do not fit (shared-memory
// window too large) are skipped. Uses only the public entry points.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/tristan_gpu.h"

namespace {
struct Cand {
    int tx, ty, tz, sort_every;
};
}  // namespace

extern "C" int tg_autotune(tg_config *cfg, void *p, int32_t ions, int32_t lecs, int32_t laps, float *best_ms,
                           float *table, int32_t table_len) {
    if (!cfg || !p || laps < 1) return -TG_ERR_ARG;
    std::vector<Cand> cands;
    const int ses[3] = {1, 2, 3};
    if (cfg->dims == 2) {
        const int tiles[5][2] = {{16, 16}, {32, 16}, {16, 32}, {32, 32}, {8, 8}};
        for (auto &t : tiles)
            for (int se : ses) cands.push_back({t[0], t[1], 1, se});
    } else {
        const int tiles[4][3] = {{8, 8, 8}, {8, 8, 4}, {16, 8, 4}, {4, 4, 4}};
        for (auto &t : tiles)
            for (int se : ses) cands.push_back({t[0], t[1], t[2], se});
    }
    float best = 1e30f;
    Cand bestc = cands[0];
    int row = 0;
    for (const Cand &c : cands) {
        tg_config t = *cfg;
        t.tile[0] = c.tx;
        t.tile[1] = c.ty;
        t.tile[2] = c.tz;
        t.sort_every = c.sort_every;
        tg_ctx *ctx = nullptr;
        if (tg_init(&t, &ctx) != TG_OK) continue;  // window does not fit, or no memory
        int32_t ni = ions, nl = lecs;
        float ms = -1.0f;
        if (tg_bind_particles(ctx, p, &ni, &nl) == TG_OK && tg_sync_from_host(ctx, TG_SYNC_PARTICLES) == TG_OK &&
            tg_step(ctx, 2 * c.sort_every) == TG_OK && tg_synchronize(ctx) == TG_OK &&
            tg_step_timed(ctx, laps * 2 * c.sort_every, &ms) == TG_OK) {
            ms /= (float)(laps * 2 * c.sort_every);
            if (ms < best) {
                best = ms;
                bestc = c;
            }
        }
        tg_finalize(ctx);
        if (table && row < table_len) {
            table[5 * row + 0] = (float)c.tx;
            table[5 * row + 1] = (float)c.ty;
            table[5 * row + 2] = (float)c.tz;
            table[5 * row + 3] = (float)c.sort_every;
            table[5 * row + 4] = ms;
            row++;
        }
    }
    if (best >= 1e30f) return -TG_ERR_STATE;
    cfg->tile[0] = bestc.tx;
    cfg->tile[1] = bestc.ty;
    cfg->tile[2] = bestc.tz;
    cfg->sort_every = bestc.sort_every;
    if (best_ms) *best_ms = best;
    return row;
}
