// Reference-style frame through the VolumeGVDB facade (include/gbvdb_volume.hpp):
// the call sequence of source/gFluidSurface/main_fluid_surface.cpp:325-356.
// Usage: facade_sample <points.f32> <radius> <mode: density|levelset>
// Prints: leaves, used leaves, subcell list length, FP64 checksum.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gbvdb_volume.hpp"

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    std::vector<float> pts;
    float buf[3];
    while (std::fread(buf, sizeof(float), 3, f) == 3) pts.insert(pts.end(), buf, buf + 3);
    std::fclose(f);
    int n = (int)(pts.size() / 3);
    float radius = (float)std::atof(argv[2]);
    bool levelset = std::strcmp(argv[3], "levelset") == 0;

    void* dpos = nullptr;
    if (cudaMalloc(&dpos, pts.size() * sizeof(float)) != cudaSuccess) return 3;
    cudaMemcpy(dpos, pts.data(), pts.size() * sizeof(float), cudaMemcpyHostToDevice);

    gbvdb::VolumeGVDB gvdb;
    gvdb.SetCudaDevice(0);
    gvdb.Initialize();
    gvdb.Configure(3, 3, 3, 3, 4);  // 5 levels, as the samples configure
    gvdb.SetChannelDefault(16, 16, 1);
    gvdb.AddChannel(0, gbvdb::T_FLOAT, 1);
    gbvdb::DataPtr pos, none;
    gvdb.SetDataGPU(pos, n, dpos, 0, 12);
    gvdb.SetPoints(pos, none, none);
    gbvdb::Vector3DF orig(0, 0, 0);
    gvdb.RebuildTopology(n, radius, orig);
    gvdb.FinishTopology(false, true);
    gvdb.UpdateAtlas();
    int len = 0;
    gvdb.InsertPointsSubcell(4, n, radius, orig, len);
    if (levelset)
        gvdb.GatherLevelSet(4, n, radius, orig, len, 0, 1);
    else
        gvdb.GatherDensity(4, n, radius, orig, len, 0, 1);
    gvdb.UpdateApron(0, levelset ? 3.0f : 0.0f);
    double sum = 0;
    gbvdb_checksum(gvdb.handle(), 0, &sum);
    std::printf("%llu %llu %d %.17g\n", (unsigned long long)gvdb.getNumTotalNodes(0),
                (unsigned long long)gvdb.getNumUsedNodes(0), len, sum);
    cudaFree(dpos);
    return gvdb.last_status() == GBVDB_OK ? 0 : 1;
}
