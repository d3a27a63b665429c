// Test infrastructure only: runs the reference's face boundary setup
// (src/setBoundaryConditions.hpp, spliced into main as ns.cpp:162 does) for face
// settings given on the command line and dumps boundary1/2/3 and u0/v0/w0, plus the
// face flag of ns.cpp:164-177, so the host case builder can be pinned to them.
//
// usage: case_ref nx ny nz  then 6 faces (nxMin nxMax nyMin nyMax nzMin nzMax) x
//        (b1 b2 b3 u0 v0 w0)  then out_prefix
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "base.hpp"

template <class T>
static void dump(const std::string& path, const std::vector<T>& v)
{
    std::ofstream o(path, std::ios::binary);
    o.write(reinterpret_cast<const char*>(v.data()), sizeof(T) * v.size());
}

int main(int argc, char** argv)
{
    if (argc != 3 + 1 + 36 + 1) return 2;
    int a = 1;
    const int nx = std::atoi(argv[a++]), ny = std::atoi(argv[a++]), nz = std::atoi(argv[a++]);
    int B[6][3];
    float U[6][3];
    for (int f = 0; f < 6; f++) {
        for (int d = 0; d < 3; d++) B[f][d] = std::atoi(argv[a++]);
        for (int d = 0; d < 3; d++) U[f][d] = std::strtof(argv[a++], nullptr);
    }
    const std::string out = argv[a++];
    int nxMinBoundary1 = B[0][0], nxMinBoundary2 = B[0][1], nxMinBoundary3 = B[0][2];
    float nxMinU0 = U[0][0], nxMinV0 = U[0][1], nxMinW0 = U[0][2];
    int nxMaxBoundary1 = B[1][0], nxMaxBoundary2 = B[1][1], nxMaxBoundary3 = B[1][2];
    float nxMaxU0 = U[1][0], nxMaxV0 = U[1][1], nxMaxW0 = U[1][2];
    int nyMinBoundary1 = B[2][0], nyMinBoundary2 = B[2][1], nyMinBoundary3 = B[2][2];
    float nyMinU0 = U[2][0], nyMinV0 = U[2][1], nyMinW0 = U[2][2];
    int nyMaxBoundary1 = B[3][0], nyMaxBoundary2 = B[3][1], nyMaxBoundary3 = B[3][2];
    float nyMaxU0 = U[3][0], nyMaxV0 = U[3][1], nyMaxW0 = U[3][2];
    int nzMinBoundary1 = B[4][0], nzMinBoundary2 = B[4][1], nzMinBoundary3 = B[4][2];
    float nzMinU0 = U[4][0], nzMinV0 = U[4][1], nzMinW0 = U[4][2];
    int nzMaxBoundary1 = B[5][0], nzMaxBoundary2 = B[5][1], nzMaxBoundary3 = B[5][2];
    float nzMaxU0 = U[5][0], nzMaxV0 = U[5][1], nzMaxW0 = U[5][2];
    (void)nxMinBoundary2; (void)nxMinBoundary3; (void)nxMaxBoundary2; (void)nxMaxBoundary3;
    (void)nyMinBoundary1; (void)nyMinBoundary3; (void)nyMaxBoundary1; (void)nyMaxBoundary3;
    (void)nzMinBoundary1; (void)nzMinBoundary2; (void)nzMaxBoundary1; (void)nzMaxBoundary2;
    const int E = nx * ny * nz;
    std::vector<float> u0(E, 0.f), v0(E, 0.f), w0(E, 0.f);
    std::vector<int> boundary(E, 0), boundary1(E, 0), boundary2(E, 0), boundary3(E, 0);
#include "setBoundaryConditions.hpp"
    // face flag: every domain-face cell, z faces only when nz > 1
    for (int ic = 0; ic < E; ic++) {
        const int i = ic2i(ic, nx, ny), j = ic2j(ic, nx, ny), k = ic2k(ic, nx, ny);
        const bool onz = (nz - 1 != 0) && (k == 0 || k == nz - 1);
        if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || onz) boundary[ic] = 1;
    }
    dump(out + "boundary.i32", boundary);
    dump(out + "boundary1.i32", boundary1);
    dump(out + "boundary2.i32", boundary2);
    dump(out + "boundary3.i32", boundary3);
    dump(out + "u0.f32", u0);
    dump(out + "v0.f32", v0);
    dump(out + "w0.f32", w0);
    return 0;
}
