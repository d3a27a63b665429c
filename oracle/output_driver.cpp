// Test infrastructure only: runs the reference's own output step (D3Q<Q>_opencl/write.hpp, the
// block ns.cpp includes after a time step) on arrays read from files, so that the device output
// reductions, the VTK writer and the restart writer can be checked against what it writes.
// The OpenCL downloads at the top of write.hpp become no-ops (cl::copy below): the host arrays
// already hold the values a download would bring.
//
// usage: output_ref<Q> in_dir work_dir nx ny nz nt dpdx c L uMax Dref forceCoeffs writeBinary
//                      outInterval timeMean
// in_dir holds raw arrays (cell order ic, populations q-major): f.f32, tauSGS.f32, omega.f32,
// Fwx.f32 Fwy.f32 Fwz.f32, GxIBM.f32 GyIBM.f32 GzIBM.f32, boundary1.i32 boundary2.i32
// boundary3.i32, sdf.f32, solid.u8, neiSolid.u8, uMean.f32 vMean.f32 wMean.f32 (the means before
// this output).  write.hpp writes ./out/resNNNNNNNN.vtk and ./out/data.dat relative to work_dir;
// this driver adds work_dir/{rho,u,v,w,uMean,vMean,wMean}.f32 and work_dir/scalars.txt
// (rho_av timeMean, both %.9g) and leaves write.hpp's own console report on stdout.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <unistd.h>

#if OUT_Q == 27
#include "D3Q27.hpp"
#else
#include "D3Q19.hpp"
#endif

namespace cl {
struct Stub {};
template <class It>
void copy(Stub&, Stub&, It, It)
{
}
}  // namespace cl

template <class T>
static std::vector<T> load(const std::string& path, size_t n)
{
    std::vector<T> v(n);
    std::ifstream in(path, std::ios::binary);
    if (!in.read(reinterpret_cast<char*>(v.data()), sizeof(T) * n)) {
        std::fprintf(stderr, "cannot read %s\n", path.c_str());
        std::exit(2);
    }
    return v;
}

template <class T>
static void dump(const std::string& path, const std::vector<T>& v)
{
    std::ofstream o(path, std::ios::binary);
    o.write(reinterpret_cast<const char*>(v.data()), sizeof(T) * v.size());
}

int main(int argc, char** argv)
{
    if (argc != 16) {
        std::fprintf(stderr,
                     "usage: %s in_dir work_dir nx ny nz nt dpdx c L uMax Dref forceCoeffs writeBinary outInterval "
                     "timeMean\n",
                     argv[0]);
        return 2;
    }
    const std::string in = std::string(argv[1]) + "/";
    const std::string work = argv[2];
    int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]), nz = std::atoi(argv[5]);
    int nt = std::atoi(argv[6]);
    float dpdx = std::strtof(argv[7], nullptr);
    const float c = std::strtof(argv[8], nullptr);
    const float L = std::strtof(argv[9], nullptr);
    float uMax = std::strtof(argv[10], nullptr);
    float Dref = std::strtof(argv[11], nullptr);
    bool forceCoeffs = std::atoi(argv[12]) != 0;
    bool writeBinary = std::atoi(argv[13]) != 0;
    int outInterval = std::atoi(argv[14]);
    float timeMean = std::strtof(argv[15], nullptr);
    const int Q = OUT_Q;
    const int elements = nx * ny * nz;
    const size_t E = (size_t)elements;

    bool Fwrite = true;
    int nextOutTime = nt;
    int startTimeStep = 0;
    const float deltaT = L / c;
    const std::vector<float> cx = setCx();
    const std::vector<float> cy = setCy();
    const std::vector<float> cz = setCz();
    std::vector<float> f = load<float>(in + "f.f32", E * Q);
    std::vector<float> tauSGS = load<float>(in + "tauSGS.f32", E);
    std::vector<float> omega = load<float>(in + "omega.f32", E);
    std::vector<float> Fwx = load<float>(in + "Fwx.f32", E), Fwy = load<float>(in + "Fwy.f32", E),
                       Fwz = load<float>(in + "Fwz.f32", E);
    std::vector<float> GxIBM = load<float>(in + "GxIBM.f32", E), GyIBM = load<float>(in + "GyIBM.f32", E),
                       GzIBM = load<float>(in + "GzIBM.f32", E);
    std::vector<int> boundary1 = load<int>(in + "boundary1.i32", E), boundary2 = load<int>(in + "boundary2.i32", E),
                     boundary3 = load<int>(in + "boundary3.i32", E);
    std::vector<float> sdf = load<float>(in + "sdf.f32", E);
    std::vector<unsigned char> solid = load<unsigned char>(in + "solid.u8", E);
    std::vector<unsigned char> neiSolid = load<unsigned char>(in + "neiSolid.u8", E);
    std::vector<float> uMean = load<float>(in + "uMean.f32", E), vMean = load<float>(in + "vMean.f32", E),
                       wMean = load<float>(in + "wMean.f32", E);
    std::vector<float> rho(E), u(E), v(E), w(E);
    float rho_av = 1.0;
    cl::Stub queue, f_d, tauSGS_d, omega_d, Fwx_d, Fwy_d, Fwz_d, GxIBM_d, GyIBM_d, GzIBM_d;
    auto start = std::chrono::system_clock::now();
    auto end = start;

    if (chdir(work.c_str()) != 0) {
        std::fprintf(stderr, "cannot enter %s\n", work.c_str());
        return 2;
    }
#include "write.hpp"

    dump("rho.f32", rho);
    dump("u.f32", u);
    dump("v.f32", v);
    dump("w.f32", w);
    dump("uMean.f32", uMean);
    dump("vMean.f32", vMean);
    dump("wMean.f32", wMean);
    std::ofstream s("scalars.txt");
    char buf[128];
    std::snprintf(buf, sizeof buf, "%.9g %.9g\n", (double)rho_av, (double)timeMean);
    s << buf;
    return 0;
}
