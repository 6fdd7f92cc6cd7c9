// gbo_launch_table.h -- tuned launch shapes per size class, measured on GB300.
//
// Written by `python -m oceananigans_gb300.autotune --write` (the fastest of a sweep of
// shapes per kernel group, timed with CUDA events); a model whose (Nx, Ny, Nz, float
// type, immersed) is listed starts from its entry, any other from the default rule.
#pragma once

struct LaunchShapeEntry {
    int nx, ny, nz, fp64, ibg;
    int dct_columns, x_lines, y_columns, levels;
};

// BEGIN TABLE
static const LaunchShapeEntry kLaunchTable[] = {
    {256, 256, 128, 0, 0, 32, 8, 8, 24},  // rect
    {256, 256, 128, 1, 0, 4, 8, 2, 24},  // rect
    {256, 256, 128, 0, 1, 32, 8, 8, 24},  // ibg
    {512, 512, 256, 0, 0, 32, 8, 8, 32},  // stretched
    {128, 128, 1, 1, 0, 32, 2, 2, 1},  // flat
    {64, 64, 32, 0, 0, 32, 4, 4, 2},  // rect
    {64, 64, 48, 0, 0, 8, 8, 4, 2},  // rect
    {64, 64, 64, 0, 0, 16, 32, 8, 4},  // rect
    {96, 96, 32, 0, 0, 32, 8, 4, 4},  // rect
    {96, 96, 48, 0, 0, 16, 8, 8, 4},  // rect
    {96, 96, 64, 0, 0, 8, 8, 8, 8},  // rect
    {128, 128, 32, 0, 0, 32, 4, 4, 8},  // rect
    {128, 128, 48, 0, 0, 32, 8, 8, 8},  // rect
    {128, 128, 64, 0, 0, 64, 8, 8, 4},  // rect
    {0, 0, 0, 0, 0, 0, 0, 0, 0},  // end
};
// END TABLE

inline const LaunchShapeEntry* tuned_shape(int nx, int ny, int nz, bool fp64, bool ibg) {
    for (const LaunchShapeEntry* e = kLaunchTable; e->nx; ++e)
        if (e->nx == nx && e->ny == ny && e->nz == nz && e->fp64 == (int)fp64 && e->ibg == (int)ibg) return e;
    return nullptr;
}
