// Frame and state files of the reference driver, from and to a GPU context.
//
//   mpmg_write_frame   the rows of write_frame / write_particle
//                      (src/writer.c:169-201): one header line
//                      "frame t num_particles", then per particle
//                      m v x y x_t y_t sxx sxy syy ux uy state[9] color
//                      state[10] active and the eight CPDI corner
//                      coordinates, in "%lg", so framereader.py and the
//                      reference's post-processing read it unchanged.  The
//                      fields come from one batched device read
//                      (mpmg_get_fields); the text is formatted by several
//                      host threads.
//   mpmg_write_state   write_state (src/writer.c:266-380), with every value
//                      in "%.17g" so that a restart is exact (the
//                      reference's "%lg" keeps six digits).
//   mpmg_read_state    read_state (src/reader.c:123-243) into a new context.
//                      The reference's reader never allocates job->active
//                      before filling it; here the activity comes with the
//                      particles.  Time and step count are restored, so the
//                      next step's body force is the one the saved run would
//                      have used.
//
// mpm_init sets color to 0, the deformation gradient to the identity and the
// CPDI corners to 0, and the USL step never changes them
// (process_usl.c:97-125), so the files carry those values.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <thread>
#include <vector>

#include "mpmg_internal.cuh"

namespace {

// A field of the context, or zeros where the context does not hold it (the
// transients of a run that does not store them, state slots the material
// does not use, or fields the mixed form does not keep).
int field_or_zero(mpmg_ctx *ctx, const char *name, std::vector<double> &out, size_t count)
{
    out.assign(count, 0.0);
    if (count == 0) return MPMG_OK;
    const int rc = mpmg_get_field(ctx, name, out.data());
    if (rc == MPMG_ERR_UNKNOWN_FIELD) {
        out.assign(count, 0.0);
        return MPMG_OK;
    }
    return rc;
}

// Formats rows [k0, k1) with fmt_row into one string per thread, then
// writes them in order.
template <typename F>
int write_rows(FILE *fd, size_t count, F fmt_row)
{
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 1;
    if (nt > 32) nt = 32;
    if (count < 4096) nt = 1;
    std::vector<std::string> parts(nt);
    std::vector<std::thread> team;
    for (unsigned t = 0; t < nt; t++) {
        const size_t k0 = count * t / nt, k1 = count * (t + 1) / nt;
        auto body = [&, t, k0, k1]() {
            std::string &s = parts[t];
            s.reserve((k1 - k0) * 160);
            char line[1024];
            for (size_t k = k0; k < k1; k++) {
                const int len = fmt_row(k, line, sizeof(line));
                if (len > 0) s.append(line, (size_t)len < sizeof(line) ? (size_t)len : sizeof(line) - 1);
            }
        };
        if (nt == 1) body();
        else team.emplace_back(body);
    }
    for (auto &th : team) th.join();
    for (auto &s : parts)
        if (!s.empty() && fwrite(s.data(), 1, s.size(), fd) != s.size()) {
            mpmg_set_error("writing the file failed");
            return MPMG_ERR_INVALID;
        }
    return MPMG_OK;
}

}  // namespace

extern "C" {

int mpmg_write_frame(mpmg_ctx *ctx, FILE *fd, size_t frame, double t)
{
    if (ctx == nullptr || fd == nullptr) return MPMG_ERR_INVALID;
    const size_t n = ctx->np;
    static const char *names[] = {"m", "v", "x", "y", "vx", "vy", "sxx", "sxy", "syy", "ux", "uy"};
    const int nf = (int)(sizeof(names) / sizeof(names[0]));
    std::vector<std::vector<double>> f(nf + 2, std::vector<double>(n ? n : 1));
    std::vector<double *> out(nf);
    for (int k = 0; k < nf; k++) out[k] = f[k].data();
    int rc = mpmg_get_fields(ctx, nf, names, out.data());
    if (rc != MPMG_OK) return rc;
    if ((rc = field_or_zero(ctx, "state9", f[nf], n)) != MPMG_OK) return rc;
    if ((rc = field_or_zero(ctx, "state10", f[nf + 1], n)) != MPMG_OK) return rc;
    std::vector<int> elem(n ? n : 1), active(n ? n : 1);
    if ((rc = mpmg_get_map(ctx, elem.data(), active.data())) != MPMG_OK) return rc;
    fprintf(fd, "%zu %lg %zu\n", frame, t, n);
    rc = write_rows(fd, n, [&](size_t i, char *buf, size_t cap) {
        // write_particle (src/writer.c:169-186): color, then the corners, are 0
        return snprintf(buf, cap,
                        "%lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg"
                        " %lg %lg %lg %lg %lg %lg %lg %lg\n",
                        f[0][i], f[1][i], f[2][i], f[3][i], f[4][i], f[5][i], f[6][i], f[7][i], f[8][i], f[9][i],
                        f[10][i], f[nf][i], 0.0, f[nf + 1][i], (double)active[i], 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
                        0.0, 0.0);
    });
    if (rc != MPMG_OK) return rc;
    fflush(fd);
    return MPMG_OK;
}

// write_element_frame (src/writer.c:205-263): per element the
// volume-weighted mean stress of its active particles, summed in particle
// order as the reference does (from one read-back of v, the stresses and the
// element map), with the element's corner coordinates (node_number_to_coords,
// element.c:10-19).
int mpmg_write_element_frame(mpmg_ctx *ctx, FILE *fd, size_t frame, double t)
{
    if (ctx == nullptr || fd == nullptr) return MPMG_ERR_INVALID;
    if (ctx->batch) {
        mpmg_set_error("element frames hold one simulation");
        return MPMG_ERR_UNSUPPORTED;
    }
    const size_t n = ctx->np, ne = ctx->ne;
    static const char *names[] = {"v", "sxx", "sxy", "syy"};
    std::vector<std::vector<double>> f(4, std::vector<double>(n ? n : 1));
    std::vector<double *> out(4);
    for (int k = 0; k < 4; k++) out[k] = f[k].data();
    int rc = mpmg_get_fields(ctx, 4, names, out.data());
    if (rc != MPMG_OK) return rc;
    std::vector<int> elem(n ? n : 1), active(n ? n : 1);
    if ((rc = mpmg_get_map(ctx, elem.data(), active.data())) != MPMG_OK) return rc;
    std::vector<double> sxx_acc(ne, 0.0), sxy_acc(ne, 0.0), syy_acc(ne, 0.0), v_acc(ne, 0.0);
    for (size_t i = 0; i < n; i++) {
        if (active[i] == 0) continue;
        const int e = elem[i];
        if (e < 0 || (size_t)e >= ne) continue;
        sxx_acc[e] += f[0][i] * f[1][i];
        sxy_acc[e] += f[0][i] * f[2][i];
        syy_acc[e] += f[0][i] * f[3][i];
        v_acc[e] += f[0][i];
    }
    const int N = ctx->cfg.Nx, Ex = N - 1;
    const double h = ctx->cfg.h;
    fprintf(fd, "%zu %lg %zu\n", frame, t, ne);
    rc = write_rows(fd, ne, [&](size_t e, char *buf, size_t cap) {
        const int n0 = (int)(e / (size_t)Ex) * N + (int)(e % (size_t)Ex);
        const int nodes[4] = {n0, n0 + 1, n0 + 1 + N, n0 + N};
        double c[8];
        for (int k = 0; k < 4; k++) {
            c[2 * k] = (nodes[k] % N) * h;
            c[2 * k + 1] = (nodes[k] / N) * h;
        }
        const double va = v_acc[e];
        return snprintf(buf, cap, "%lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg\n", c[0], c[1], c[2], c[3], c[4],
                        c[5], c[6], c[7], (va > 0) ? (sxx_acc[e] / va) : 0.0f, (va > 0) ? (sxy_acc[e] / va) : 0.0f,
                        (va > 0) ? (syy_acc[e] / va) : 0.0f);
    });
    if (rc != MPMG_OK) return rc;
    fflush(fd);
    return MPMG_OK;
}

int mpmg_write_state(mpmg_ctx *ctx, FILE *fd, double t_stop)
{
    if (ctx == nullptr || fd == nullptr) return MPMG_ERR_INVALID;
    const size_t n = ctx->np;
    if (ctx->batch) {
        mpmg_set_error("state files hold one simulation");
        return MPMG_ERR_UNSUPPORTED;
    }
    static const char *names[] = {"x", "y", "vx", "vy", "m", "v", "sxx", "sxy", "syy", "ux", "uy"};
    const int nf = (int)(sizeof(names) / sizeof(names[0]));
    std::vector<std::vector<double>> f(nf, std::vector<double>(n ? n : 1));
    std::vector<double *> out(nf);
    for (int k = 0; k < nf; k++) out[k] = f[k].data();
    int rc = mpmg_get_fields(ctx, nf, names, out.data());
    if (rc != MPMG_OK) return rc;
    std::vector<double> v0, exx, exy, eyy, wxy, by;
    if ((rc = field_or_zero(ctx, "v0", v0, n)) != MPMG_OK) return rc;
    if (ctx->mixed) v0 = f[5];     // the mixed form keeps no initial volume
    if ((rc = field_or_zero(ctx, "exx", exx, n)) != MPMG_OK) return rc;
    if ((rc = field_or_zero(ctx, "exy", exy, n)) != MPMG_OK) return rc;
    if ((rc = field_or_zero(ctx, "eyy", eyy, n)) != MPMG_OK) return rc;
    if ((rc = field_or_zero(ctx, "wxy", wxy, n)) != MPMG_OK) return rc;
    if ((rc = field_or_zero(ctx, "by", by, n)) != MPMG_OK) return rc;
    std::vector<std::vector<double>> st(MPMG_DEPVAR);
    for (int k = 0; k < MPMG_DEPVAR; k++) {
        char name[16];
        snprintf(name, sizeof(name), "state%d", k);
        if ((rc = field_or_zero(ctx, name, st[k], n)) != MPMG_OK) return rc;
    }
    // The file has no place for g_local_mu2's out-of-plane stress T[ZZ]; it
    // travels in state[8], a slot that material zeroes at material_init and
    // never reads (g_local_mu2.c:53, :106-125).
    if (ctx->cfg.material == MPMG_G_LOCAL_MU2 && (rc = field_or_zero(ctx, "Tzz", st[8], n)) != MPMG_OK) return rc;
    std::vector<int> elem(n ? n : 1), active(n ? n : 1);
    if ((rc = mpmg_get_map(ctx, elem.data(), active.data())) != MPMG_OK) return rc;
    double t = 0;
    if ((rc = mpmg_get_time(ctx, &t, nullptr)) != MPMG_OK && rc != MPMG_ERR_SOLVER) return rc;
    const int N = ctx->cfg.Nx;
    const double h = ctx->cfg.h;
    if (ctx->cfg.Nx != ctx->cfg.Ny) {
        mpmg_set_error("state files describe square N x N grids");
        return MPMG_ERR_UNSUPPORTED;
    }
    fprintf(fd, "%.17g %.17g %.17g\n", t, ctx->cfg.dt, t_stop);
    fprintf(fd, "%zu %zu %zu\n", n, ctx->nn, ctx->ne);
    fprintf(fd, "%d %.17g\n", N, h);
    const int Ex = ctx->Ex;
    rc = write_rows(fd, n, [&](size_t i, char *buf, size_t cap) {
        // local coordinates in the particle's element, as the step's shape
        // functions use them (zero outside the grid)
        double xl = 0, yl = 0;
        if (elem[i] >= 0) {
            xl = (f[0][i] - (elem[i] % Ex) * h) / h;
            yl = (f[1][i] - (elem[i] / Ex) * h) / h;
        }
        int len = snprintf(buf, cap,
                           "%.17g %.17g\n%.17g %.17g\n%.17g %.17g\n%.17g\n%.17g\n%.17g\n%.17g %.17g %.17g\n"
                           "%.17g %.17g %.17g %.17g\n%.17g %.17g\n1 0 0 1\n%.17g %.17g\n0\n%d\n",
                           f[0][i], f[1][i], xl, yl, f[2][i], f[3][i], f[4][i], f[5][i], v0[i], f[6][i], f[7][i],
                           f[8][i], exx[i], exy[i], eyy[i], wxy[i], 0.0, by[i], f[9][i], f[10][i], MPMG_DEPVAR);
        for (int k = 0; k < MPMG_DEPVAR && len > 0 && (size_t)len < cap; k++)
            len += snprintf(buf + len, cap - len, "%.17g\n", st[k][i]);
        if (len > 0 && (size_t)len < cap) len += snprintf(buf + len, cap - len, "%d\n", active[i]);
        return len;
    });
    if (rc != MPMG_OK) return rc;
    // nodes (node_number_to_coords, element.c:10-19) and element connectivity
    // (BL, BR, TR, TL, process_usl.c:140-143)
    rc = write_rows(fd, ctx->nn, [&](size_t k, char *buf, size_t cap) {
        return snprintf(buf, cap, "%.17g %.17g\n", (double)(k % N) * h, (double)(k / N) * h);
    });
    if (rc != MPMG_OK) return rc;
    rc = write_rows(fd, ctx->ne, [&](size_t e, char *buf, size_t cap) {
        const int c = (int)(e % (size_t)Ex), r = (int)(e / (size_t)Ex);
        const int n0 = r * N + c;
        return snprintf(buf, cap, "%d %d %d %d\n", n0, n0 + 1, n0 + N + 1, n0 + N);
    });
    if (rc != MPMG_OK) return rc;
    fflush(fd);
    return MPMG_OK;
}

int mpmg_read_state(FILE *fd, const mpmg_config *base, mpmg_ctx **out)
{
    if (fd == nullptr || base == nullptr || out == nullptr) return MPMG_ERR_INVALID;
    *out = nullptr;
    double t = 0, dt = 0, t_stop = 0, h = 0;
    size_t np = 0, nn = 0, ne = 0, N = 0;
    if (fscanf(fd, "%lg %lg %lg", &t, &dt, &t_stop) != 3 || fscanf(fd, "%zu %zu %zu", &np, &nn, &ne) != 3 ||
        fscanf(fd, "%zu %lg", &N, &h) != 2) {
        mpmg_set_error("state header unreadable");
        return MPMG_ERR_INVALID;
    }
    if (N < 2 || nn != N * N || ne != (N - 1) * (N - 1)) {
        mpmg_set_error("state header: %zu nodes and %zu elements do not make an N = %zu grid", nn, ne, N);
        return MPMG_ERR_INVALID;
    }
    std::vector<double> x(np), y(np), vx(np), vy(np), m(np), v(np), v0(np), sxx(np), sxy(np), syy(np), ux(np),
        uy(np);
    std::vector<std::vector<double>> st(MPMG_DEPVAR, std::vector<double>(np, 0.0));
    std::vector<int> active(np);
    for (size_t i = 0; i < np; i++) {
        double xl, yl, e[4], b[2], F[4], color;
        int dep = 0;
        int r = fscanf(fd, "%lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg", &x[i], &y[i], &xl, &yl, &vx[i],
                       &vy[i], &m[i], &v[i], &v0[i], &sxx[i], &sxy[i], &syy[i]);
        r += fscanf(fd, "%lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg", &e[0], &e[1], &e[2], &e[3], &b[0],
                    &b[1], &F[0], &F[1], &F[2], &F[3], &ux[i], &uy[i], &color);
        r += fscanf(fd, "%d", &dep);
        if (r != 26 || dep < 0 || dep > 64) {
            mpmg_set_error("state of particle %zu unreadable", i);
            return MPMG_ERR_INVALID;
        }
        for (int k = 0; k < dep; k++) {
            double s;
            if (fscanf(fd, "%lg", &s) != 1) {
                mpmg_set_error("state variables of particle %zu unreadable", i);
                return MPMG_ERR_INVALID;
            }
            if (k < MPMG_DEPVAR) st[k][i] = s;
        }
        if (fscanf(fd, "%d", &active[i]) != 1) {
            mpmg_set_error("activity of particle %zu unreadable", i);
            return MPMG_ERR_INVALID;
        }
    }
    // node coordinates and connectivity follow; the grid is regular, so they
    // are checked by count only
    mpmg_config cfg = *base;
    cfg.Nx = cfg.Ny = (int)N;
    cfg.h = h;
    cfg.dt = dt;
    mpmg_ctx *ctx = nullptr;
    int rc = mpmg_create(&cfg, np, m.data(), v.data(), x.data(), y.data(), vx.data(), vy.data(), sxx.data(),
                         sxy.data(), syy.data(), &ctx);
    if (rc != MPMG_OK) return rc;
    auto put = [&](const char *name, const std::vector<double> &a) {
        const int r = mpmg_set_field(ctx, name, a.data());
        return r == MPMG_ERR_UNKNOWN_FIELD ? MPMG_OK : r;   // a field this form does not hold
    };
    rc = put("ux", ux);
    if (rc == MPMG_OK) rc = put("uy", uy);
    if (rc == MPMG_OK && !ctx->mixed) rc = put("v0", v0);
    for (int k = 0; k < MPMG_DEPVAR && rc == MPMG_OK; k++) {
        char name[16];
        snprintf(name, sizeof(name), "state%d", k);
        if (cfg.material == MPMG_G_LOCAL_MU2 && k == 8) rc = put("Tzz", st[8]);   // see mpmg_write_state
        else rc = put(name, st[k]);
    }
    if (rc == MPMG_OK && !ctx->mixed) {
        // particles the saved run had retired stay retired
        std::vector<int> elem(np ? np : 1), act(np ? np : 1);
        rc = mpmg_get_map(ctx, elem.data(), act.data());
        for (size_t i = 0; i < np && rc == MPMG_OK; i++) {
            if (!active[i]) {
                act[i] = 0;
                elem[i] = -1;
            }
        }
        if (rc == MPMG_OK && np) rc = mpmg_set_map(ctx, elem.data(), act.data());
    }
    // the step count the saved time corresponds to: its sign is what the
    // body-force ramp reads (loading.c:34-54)
    if (rc == MPMG_OK) rc = mpmg_set_time(ctx, t, t > 0 ? (int)llround(t / dt) : 0);
    if (rc != MPMG_OK) {
        mpmg_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return MPMG_OK;
}

}  // extern "C"
