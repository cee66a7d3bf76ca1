// Grid geometry, boundary conditions and shape functions of the FP64 step,
// shared by the step (mpmg_step.cu) and its adjoint (mpmg_adjoint.cu).
#pragma once

#include "mpmg_internal.cuh"

namespace fp64 {

struct GridGeom {
    int Nx, Ny, Ex, Ey;
    double h, inv_h, xmax, ymax;
};

struct BcParams {
    int kind;
    // box: wall columns / rows and friction bits
    int left_col, right_col, bottom_row, top_row;
    int lf, bf, rf, tf;
    // silo
    double hole_radius, open_time;
    int wall_col;
};

struct ShapeFns {
    double s[4], gx[4], gy[4];
};

// tent and grad_tent (interpolate.c:23-65) at local coordinates (xl, yl);
// node order BL, BR, TR, TL (process_usl.c:140-143).
__device__ __forceinline__ ShapeFns shape(double xl, double yl, double inv_h)
{
    ShapeFns f;
    double ox = 1 - xl, oy = 1 - yl;
    f.s[0] = ox * oy;
    f.s[1] = xl * oy;
    f.s[2] = xl * yl;
    f.s[3] = ox * yl;
    f.gx[0] = -oy * inv_h;
    f.gx[1] = oy * inv_h;
    f.gx[2] = yl * inv_h;
    f.gx[3] = -yl * inv_h;
    f.gy[0] = -ox * inv_h;
    f.gy[1] = -xl * inv_h;
    f.gy[2] = xl * inv_h;
    f.gy[3] = ox * inv_h;
    return f;
}

__device__ __forceinline__ void bc_mask(const BcParams &bc, const GridGeom &g, int i, int j,
                                        double t_now, bool &mx, bool &my)
{
    mx = false;
    my = false;
    if (bc.kind == MPMG_BOX) {
        // box.c:106-167
        bool on_row = (i >= bc.left_col && i <= bc.right_col);
        bool on_col = (j >= bc.bottom_row && j <= bc.top_row);
        if (on_row && j == bc.bottom_row) { mx |= (bc.bf & 1) != 0; my |= (bc.bf & 2) != 0; }
        if (on_row && j == bc.top_row) { mx |= (bc.tf & 1) != 0; my |= (bc.tf & 2) != 0; }
        if (on_col && i == bc.left_col) { mx |= (bc.lf & 1) != 0; my |= (bc.lf & 2) != 0; }
        if (on_col && i == bc.right_col) { mx |= (bc.rf & 1) != 0; my |= (bc.rf & 2) != 0; }
    } else {
        // square_silo.c:58-91: floor (trapdoor open at x <= hole radius after
        // the opening time), frictionless walls at column 0 and wall_col
        if (j == 0) {
            double xnode = i * g.h;
            if (!(xnode <= bc.hole_radius && t_now > bc.open_time)) {
                mx = true;
                my = true;
            }
        }
        if (i == 0 || i == bc.wall_col) mx = true;
    }
}

inline GridGeom make_geom(const mpmg_ctx *ctx)
{
    GridGeom g;
    g.Nx = ctx->cfg.Nx;
    g.Ny = ctx->cfg.Ny;
    g.Ex = ctx->Ex;
    g.Ey = ctx->Ey;
    g.h = ctx->cfg.h;
    g.inv_h = ctx->inv_h;
    g.xmax = ctx->cfg.xmax;
    g.ymax = ctx->cfg.ymax;
    return g;
}

inline BcParams make_bc(const mpmg_ctx *ctx)
{
    BcParams b = {};
    const mpmg_config &c = ctx->cfg;
    b.kind = c.bc;
    if (c.bc == MPMG_BOX) {
        // box.c:92-95 (fractions of the grid's node span)
        b.left_col = (int)(size_t)(c.bcf[0] * (double)(c.Nx - 1));
        b.right_col = (int)(size_t)((c.bcf[0] + c.bcf[2]) * (double)(c.Nx - 1));
        b.bottom_row = (int)(size_t)(c.bcf[1] * (double)(c.Ny - 1));
        b.top_row = (int)(size_t)((c.bcf[1] + c.bcf[3]) * (double)(c.Ny - 1));
        b.lf = c.bci[0];
        b.bf = c.bci[1];
        b.rf = c.bci[2];
        b.tf = c.bci[3];
    } else {
        b.hole_radius = c.bcf[0];
        b.open_time = c.bcf[1];
        b.wall_col = (int)((double)(c.Nx - 1) * c.bcf[2]);   // square_silo.c:44
    }
    return b;
}

}  // namespace fp64
