// jt_plan_table.h -- pass split per power-of-two length, indexed by log2 n:
// {0,0,0} one pass, {a,b,0} two passes 2^a (column) x 2^b (row), {a,b,c}
// three passes, {-1,-1,-1} no entry (the engine's rules decide).
// Regenerated by `python -m jtransforms_gb300.autotune` on the target GPU;
// the measurements are in plan_table_f32.json and plan_table_f64.json.
#pragma once

static const signed char kSplitF32[31][3] = {
    {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1},
    {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {9, 6, 0},
    {9, 7, 0}, {9, 8, 0}, {10, 8, 0}, {10, 9, 0}, {10, 10, 0}, {11, 10, 0}, {11, 11, 0}, {11, 12, 0},
    {8, 9, 7}, {9, 9, 7}, {9, 9, 8}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1},
};

static const signed char kSplitF64[31][3] = {
    {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1},
    {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {7, 7, 0}, {8, 7, 0},
    {8, 8, 0}, {11, 6, 0}, {11, 7, 0}, {11, 8, 0}, {11, 9, 0}, {11, 10, 0}, {11, 11, 0}, {12, 11, 0},
    {8, 8, 8}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1}, {-1, -1, -1},
};

// Elements per CTA of the generic tile kernel (mixed-radix lengths), indexed
// by ceil(log2 L); 0: the default (4096 float, 2048 double).
static const short kTileElemsF32[14] = {0, 0, 0, 0, 512, 512, 512, 1024, 1024, 1024, 1024, 2048, 4096, 8192};
static const short kTileElemsF64[14] = {0, 0, 0, 0, 512, 512, 512, 512, 1024, 2048, 2048, 2048, 4096, 0};

// Pass order of the generic tile kernel (direct_radices' `order`), indexed by
// ceil(log2 L); 0: power-of-two radices (16s) first.
static const signed char kRadixOrderF32[14] = {0, 0, 0, 0, 1, 3, 0, 0, 2, 0, 0, 0, 0, 0};
static const signed char kRadixOrderF64[14] = {0, 0, 0, 0, 1, 1, 0, 0, 2, 0, 0, 2, 0, 0};
