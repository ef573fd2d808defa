// The on-disk formats behind the C ABI: the reference's workload snapshots (tools/benchmark/bench_common.hpp:109-134,
// a raw GpuBoid array) and its baked terrace volume (src/sdf.cpp:84-107, raw float32 res^3). Plain binary files, no
// header; sizes are checked exactly, as the reference's loaders do.
#include "../../include/swarm_cuda.h"

#include <cstdio>

namespace {

long fileBytes(const char* path) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return -1;
    long size = -1;
    if (std::fseek(f, 0, SEEK_END) == 0) size = std::ftell(f);
    std::fclose(f);
    return size;
}

int readExact(const char* path, void* out, size_t bytes) {
    if (fileBytes(path) != long(bytes)) return SWARM_E_INVALID;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return SWARM_E_INVALID;
    const size_t got = std::fread(out, 1, bytes, f);
    std::fclose(f);
    return got == bytes ? SWARM_OK : SWARM_E_INVALID;
}

}  // namespace

extern "C" int swarm_snapshot_write(const char* path, const float* boids, int n) {
    if (!path || !boids || n <= 0) return SWARM_E_INVALID;
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return SWARM_E_INVALID;
    const size_t bytes = size_t(n) * 32;
    const size_t put = std::fwrite(boids, 1, bytes, f);
    const bool ok = std::fclose(f) == 0 && put == bytes;
    return ok ? SWARM_OK : SWARM_E_INVALID;
}

extern "C" int swarm_snapshot_read(const char* path, float* boids, int n) {
    if (!path || !boids || n <= 0) return SWARM_E_INVALID;
    return readExact(path, boids, size_t(n) * 32);
}

extern "C" int swarm_snapshot_count(const char* path) {
    if (!path) return -1;
    const long b = fileBytes(path);
    if (b <= 0 || b % 32 != 0 || b / 32 > 2147483647L) return -1;
    return int(b / 32);
}

extern "C" int swarm_sdf_read(const char* path, float* sdf, int res) {
    if (!path || !sdf || res <= 1 || res > 2048) return SWARM_E_INVALID;
    return readExact(path, sdf, size_t(res) * size_t(res) * size_t(res) * sizeof(float));
}
