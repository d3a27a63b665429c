// Test infrastructure only: runs the reference's own host geometry setup
// (src/walls.hpp, src/stl.hpp) the way D3Q19_opencl/ns.cpp:189-225 does and
// dumps the arrays it produces, so the device-side flag / link-table builder
// can be checked bit-exactly against them.
//
// usage: voxel_ref<Q> walls.stl nx ny nz L invertFluidSolid withSDF
//                     bxmin bxmax bymin bymax bzmin bzmax out_prefix
// The six b* are the face BC codes used by setSDFnearBwalls (boundary1 on the
// x faces, boundary2 on the y faces, boundary3 on the z faces).
// Writes <out_prefix>solid.u8, neiSolid.u8, sdf.f32 (raw, cell order ic).
#include <algorithm>
#include <cstdio>
#include <iostream>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#if VOX_Q == 27
#include "D3Q27.hpp"
#else
#include "D3Q19.hpp"
#endif
#include "input.hpp"
#include "walls.hpp"

template <class T>
static void dump(const std::string& path, const std::vector<T>& v)
{
    std::ofstream o(path, std::ios::binary);
    o.write(reinterpret_cast<const char*>(v.data()), sizeof(T) * v.size());
}

int main(int argc, char** argv)
{
    if (argc != 15) {
        std::fprintf(stderr, "usage: %s stl nx ny nz L invert withSDF bxmin bxmax bymin bymax bzmin bzmax out\n", argv[0]);
        return 2;
    }
    const std::string stl = argv[1];
    const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
    const float L = std::strtof(argv[5], nullptr);
    const bool invert = std::atoi(argv[6]) != 0;
    const bool withSDF = std::atoi(argv[7]) != 0;
    const int bc[6] = {std::atoi(argv[8]), std::atoi(argv[9]), std::atoi(argv[10]),
                       std::atoi(argv[11]), std::atoi(argv[12]), std::atoi(argv[13])};
    const std::string out = argv[14];
    const int elements = nx * ny * nz;

    std::vector<int> boundary1(elements, 0), boundary2(elements, 0), boundary3(elements, 0);
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int ic = index1d(i, j, k, nx, ny);
                if (i == 0) boundary1[ic] = bc[0];
                else if (i == nx - 1) boundary1[ic] = bc[1];
                if (j == 0) boundary2[ic] = bc[2];
                else if (j == ny - 1) boundary2[ic] = bc[3];
                if (k == 0) boundary3[ic] = bc[4];
                else if (k == nz - 1) boundary3[ic] = bc[5];
            }

    STL wallSTL(stl, L);
    std::vector<unsigned char> solid(elements, 0);
    setSolid(solid, wallSTL, nx, ny, nz, invert);
    std::vector<unsigned char> neiSolid(elements, 0);
    setNeiSolid(neiSolid, solid, nx, ny, nz, VOX_Q);

    const float sdfIni = 10000.f;
    std::vector<float> sdf(elements, sdfIni);
    float dr = 10.f;
    const float p = 7.f;
    for (int iPatch = 0; iPatch < (int)wallSTL.patch.size(); iPatch++) {
        const std::unique_ptr<STLpatch>& patch = wallSTL.patch[iPatch];
        if (withSDF) setSDF(sdf, sdfIni, dr, p, patch, nx, ny, nz, false, neiSolid);
    }
    dr = 3.f;
    if (withSDF) setSDFnearBwalls(sdf, dr, boundary1, boundary2, boundary3, nx, ny, nz);

    dump(out + "solid.u8", solid);
    dump(out + "neiSolid.u8", neiSolid);
    dump(out + "sdf.f32", sdf);
    return 0;
}
