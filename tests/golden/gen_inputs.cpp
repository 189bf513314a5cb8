// gen_inputs.cpp -- regenerates the seeded random inputs the reference's tests
// build with std::mt19937 + std::uniform_real_distribution<float>:
//   grid_8193.bin     test/test_spatial_grid.cu:649-680   seed 0x5A17,
//                     x ~ U(-12, 13), y ~ U(-9, 11), z ~ U(-7, 10)
//   neighbors_257.bin test/test_neighbors.cu:342-358      seed 12345, U(0, 5)
// Output: little-endian float32 (x, y, z, w=1) rows.
#include <cstdio>
#include <random>
#include <vector>

static void write(const char* path, const std::vector<float>& v) {
    FILE* f = std::fopen(path, "wb");
    if (!f) { std::perror(path); std::exit(1); }
    std::fwrite(v.data(), sizeof(float), v.size(), f);
    std::fclose(f);
}

int main(int argc, char** argv) {
    const char* dir = argc > 1 ? argv[1] : ".";
    char path[4096];
    {
        std::mt19937 eng(0x5A17U);
        std::uniform_real_distribution<float> dx(-12.0f, 13.0f), dy(-9.0f, 11.0f), dz(-7.0f, 10.0f);
        std::vector<float> out;
        for (int i = 0; i < 8193; ++i) {
            const float x = dx(eng);
            const float y = dy(eng);
            const float z = dz(eng);
            out.insert(out.end(), {x, y, z, 1.0f});
        }
        std::snprintf(path, sizeof(path), "%s/grid_8193.bin", dir);
        write(path, out);
    }
    {
        std::mt19937 eng(12345);
        std::uniform_real_distribution<float> d(0.0f, 5.0f);
        std::vector<float> out;
        for (int i = 0; i < 257; ++i) {
            const float x = d(eng);
            const float y = d(eng);
            const float z = d(eng);
            out.insert(out.end(), {x, y, z, 1.0f});
        }
        std::snprintf(path, sizeof(path), "%s/neighbors_257.bin", dir);
        write(path, out);
    }
    return 0;
}
