// A compiled host for the C-ABI: the reference's main loop
// (code/tristanmainloop.F90:117-303) as a sequence of calls into
// libtristan_gpu, the way the Fortran bind(C) shim drives it, with the state
// in host arrays the caller owns.
//
//   mainloop <state-in> <state-out> <laps> [fused]
//
// A state file is the tg_config struct, the nine field arrays (ex ey ez bx
// by bz curx cury curz, mx*my*mz floats each, Fortran order), the particle
// records (2 * maxhlf records of 40 bytes: ions from 0, electrons from
// maxhlf) and the two counts (int32). With "fused" the laps run through
// tg_step_host instead of one call per subroutine.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "tristan_gpu.h"

namespace {

struct State {
    tg_config cfg;
    std::vector<float> f[9];
    std::vector<unsigned char> p;
    int32_t ions = 0, lecs = 0;
};

bool read_state(const char *path, State &s) {
    FILE *fp = fopen(path, "rb");
    if (!fp) return false;
    bool ok = fread(&s.cfg, sizeof s.cfg, 1, fp) == 1;
    const size_t lot = ok ? (size_t)s.cfg.mx * s.cfg.my * s.cfg.mz : 0;
    for (int a = 0; a < 9 && ok; a++) {
        s.f[a].resize(lot);
        ok = fread(s.f[a].data(), 4, lot, fp) == lot;
    }
    if (ok) {
        s.p.resize((size_t)s.cfg.maxhlf * 2 * 40);
        ok = fread(s.p.data(), 1, s.p.size(), fp) == s.p.size();
    }
    ok = ok && fread(&s.ions, 4, 1, fp) == 1 && fread(&s.lecs, 4, 1, fp) == 1;
    fclose(fp);
    return ok;
}

bool write_state(const char *path, const State &s) {
    FILE *fp = fopen(path, "wb");
    if (!fp) return false;
    bool ok = fwrite(&s.cfg, sizeof s.cfg, 1, fp) == 1;
    for (int a = 0; a < 9 && ok; a++) ok = fwrite(s.f[a].data(), 4, s.f[a].size(), fp) == s.f[a].size();
    ok = ok && fwrite(s.p.data(), 1, s.p.size(), fp) == s.p.size();
    ok = ok && fwrite(&s.ions, 4, 1, fp) == 1 && fwrite(&s.lecs, 4, 1, fp) == 1;
    return fclose(fp) == 0 && ok;
}

// the shim's check: print the library's message and stop, as the reference
// does on its own errors
void check(tg_ctx *ctx, int rc, const char *what) {
    if (rc == TG_OK) return;
    fprintf(stderr, "%s: error %d: %s\n", what, rc, tg_last_error(ctx));
    exit(2);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s <state-in> <state-out> <laps> [fused]\n", argv[0]);
        return 1;
    }
    State s;
    if (!read_state(argv[1], s)) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 1;
    }
    const int laps = atoi(argv[3]);
    const bool fused = argc > 4 && strcmp(argv[4], "fused") == 0;
    tg_ctx *ctx = nullptr;
    check(nullptr, tg_init(&s.cfg, &ctx), "tg_init");
    check(ctx, tg_bind_fields(ctx, s.f[0].data(), s.f[1].data(), s.f[2].data(), s.f[3].data(), s.f[4].data(),
                              s.f[5].data(), s.f[6].data(), s.f[7].data(), s.f[8].data()),
          "tg_bind_fields");
    check(ctx, tg_bind_particles(ctx, s.p.data(), &s.ions, &s.lecs), "tg_bind_particles");
    if (fused) {
        check(ctx, tg_step_host(ctx, laps), "tg_step_host");
    } else {
        check(ctx, tg_sync_from_host(ctx, TG_SYNC_ALL), "tg_sync_from_host");
        for (int lap = 1; lap <= laps; lap++) {
            check(ctx, tg_bc_b1(ctx), "bc_b1");
            check(ctx, tg_bc_e1(ctx), "bc_e1");
            check(ctx, tg_advance_b_half(ctx), "advance_Bhalfstep");
            check(ctx, tg_bc_b1(ctx), "bc_b1");
            check(ctx, tg_move(ctx), "move_particles");
            check(ctx, tg_advance_b_half(ctx), "advance_Bhalfstep");
            check(ctx, tg_bc_b1(ctx), "bc_b1");
            check(ctx, tg_bc_b1(ctx), "bc_b2");
            check(ctx, tg_advance_e(ctx), "advance_Efield");
            check(ctx, tg_bc_e1(ctx), "bc_e2");
            check(ctx, tg_reset_currents(ctx), "reset_currents");
            check(ctx, tg_bc_e1(ctx), "bc_e1");
            check(ctx, tg_bc_b1(ctx), "bc_b1");
            check(ctx, tg_deposit(ctx), "deposit_particles");
            check(ctx, tg_fold_currents(ctx), "exchange_current");
            check(ctx, tg_filter(ctx), "apply_filter1_opt");
            check(ctx, tg_add_current(ctx), "add_current");
            check(ctx, tg_reorder(ctx, lap, 0), "reorder_particles");
        }
        check(ctx, tg_sync_to_host(ctx, TG_SYNC_ALL), "tg_sync_to_host");
    }
    tg_finalize(ctx);
    if (!write_state(argv[2], s)) {
        fprintf(stderr, "cannot write %s\n", argv[2]);
        return 1;
    }
    return 0;
}
