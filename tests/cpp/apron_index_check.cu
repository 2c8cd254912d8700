// Host-side check of the apron record index math shared by the apron kernels and
// the gather's fused apron (gvdb-voxels_gb300/csrc/common.cuh): apron_shell_pos is
// the inverse of apron_index over the 1,736 apron voxels of a padded 18^3 brick, and
// the edge/corner table names, for each record, the source voxel and the receiving
// direction that apron_index implies.  Runs on the host only; prints "ok".
#include <cstdio>

#include "common.cuh"

using namespace gbvdb;

int main() {
    int bad = 0, shell = 0;
    static int seen[1736] = {0};
    for (int z = 0; z < 18; z++)
        for (int y = 0; y < 18; y++)
            for (int x = 0; x < 18; x++) {
                const bool on = x == 0 || x == 17 || y == 0 || y == 17 || z == 0 || z == 17;
                if (!on) continue;
                shell++;
                const int k = apron_index(x, y, z);
                if (k < 0 || k >= 1736) { bad++; continue; }
                seen[k]++;
                int px, py, pz;
                apron_shell_pos(k, px, py, pz);
                if (px != x || py != y || pz != z) bad++;
            }
    for (int k = 0; k < 1736; k++) if (seen[k] != 1) bad++;
    // edge / corner table: record 1536 + j comes from the source voxel it names, and the
    // receiver lies in the direction opposite to where the voxel sits on the shell
    const ApronEdgeTable t = make_apron_edge_table();
    for (int j = 0; j < 200; j++) {
        int x, y, z;
        apron_shell_pos(1536 + j, x, y, z);
        const int dx = x == 0 ? -1 : (x == 17 ? 1 : 0), dy = y == 0 ? -1 : (y == 17 ? 1 : 0),
                  dz = z == 0 ? -1 : (z == 17 ? 1 : 0);
        const unsigned src = t.e[j] & 4095u, recv = t.e[j] >> 12;
        const int sx = x - 1 - 16 * dx, sy = y - 1 - 16 * dy, sz = z - 1 - 16 * dz;
        if (sx < 0 || sx > 15 || sy < 0 || sy > 15 || sz < 0 || sz > 15) bad++;
        if (src != (unsigned)((sz << 8) | (sy << 4) | sx)) bad++;
        if (recv != (unsigned)((1 - dz) * 9 + (1 - dy) * 3 + (1 - dx))) bad++;
        if ((dx != 0) + (dy != 0) + (dz != 0) < 2) bad++;  // records 1536+ are edges and corners
    }
    if (shell != 1736) bad++;
    printf("%s %d\n", bad ? "bad" : "ok", bad);
    return bad ? 1 : 0;
}
