// swgb_raster.cu -- the raster kernel variants of one colour format
// (SWGB_RASTER_CF = 0 R8G8B8A8_UNORM, 1 R16G16B16A16_SFLOAT,
// 2 R32G32B32A32_SFLOAT, 3 B8G8R8A8_UNORM): every bin shape, with and without
// hierarchical depth rejection, single-sample and (16x16 bins) four-sample,
// for the common pixel pipeline; 16x16 bins for the full one (D16_UNORM
// depth, depth bias, depth bounds, stencil).  The build compiles
// this file once per format, in parallel, and links the objects into libswgb.
#define SWGB_RASTER_TU 1
#include "swgb_kernels.cuh"

#ifndef SWGB_RASTER_CF
#error "SWGB_RASTER_CF (colour format index) must be defined"
#endif

namespace swgbk {

namespace {

template<int CF, int MS, int BW, int BH, bool HIZ, bool FULL>
void launch_raster_t(const DrawParams &D, uint32_t blocks, cudaStream_t st)
{
    k_raster<CF, MS, BW, BH, HIZ, FULL><<<blocks, RASTER_THREADS, raster_smem<CF, MS, BW, BH, FULL>(), st>>>(D);
}

template<int CF, int MS, int BW, int BH, bool HIZ, bool FULL>
void launch_raster_batch_t(const BatchPtrs &P, uint32_t blocks, cudaStream_t st)
{
    k_raster_batch<CF, MS, BW, BH, HIZ, FULL><<<blocks, RASTER_THREADS, raster_smem<CF, MS, BW, BH, FULL>(), st>>>(P);
}

template<int CF, int MS, int BW, int BH, bool HIZ, bool FULL = false>
void put(RasterKernel *table)
{
    table[raster_index(shape_index(BW, BH), HIZ, MS, CF, FULL)] = {
        (const void *)k_raster<CF, MS, BW, BH, HIZ, FULL>, (const void *)k_raster_batch<CF, MS, BW, BH, HIZ, FULL>,
        raster_smem<CF, MS, BW, BH, FULL>(), launch_raster_t<CF, MS, BW, BH, HIZ, FULL>, launch_raster_batch_t<CF, MS, BW, BH, HIZ, FULL>};
}

}  // namespace

template<>
void fill_raster_table<SWGB_RASTER_CF>(RasterKernel *table)
{
    constexpr int CF = SWGB_RASTER_CF;
    put<CF, 1, 16, 16, true>(table);
    put<CF, 1, 16, 16, false>(table);
    put<CF, 1, 32, 16, true>(table);
    put<CF, 1, 32, 16, false>(table);
    put<CF, 1, 32, 32, true>(table);
    put<CF, 1, 32, 32, false>(table);
    put<CF, 4, 16, 16, true>(table);
    put<CF, 4, 16, 16, false>(table);
    put<CF, 1, 16, 16, true, true>(table);
    put<CF, 1, 16, 16, false, true>(table);
    put<CF, 4, 16, 16, true, true>(table);
    put<CF, 4, 16, 16, false, true>(table);
    static_assert(NSHAPES == 3 && NRASTER == NSHAPES * 2 * NCF + 2 * NCF + 4 * NCF, "one entry per shape, hiz, samples and pixel pipeline");
}

}  // namespace swgbk
