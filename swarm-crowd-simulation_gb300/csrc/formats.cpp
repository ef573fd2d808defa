// The on-disk formats behind the C ABI: the reference's workload snapshots (tools/benchmark/bench_common.hpp:109-134,
// a raw GpuBoid array) and its baked terrace volume (src/sdf.cpp:84-107, raw float32 res^3): plain binary files, no
// header, sizes checked exactly as the reference's loaders do; and its navigation-field cache files (nav::save /
// nav::load, src/nav_field.cpp:554-656), read into the GPU table of the seated venues.
#include "../../include/swarm_cuda.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

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

// ---- the navigation-field cache (src/nav_field.cpp:554-656) ----
// "SWNAVF01" | payload: version u32, res u32, origin f32, cell f32, invCell f32, exits u32, key u64, then per cell
// floorZ f32, cls u8, out u8, exitRegion i8, dist f32, anchor i32, exitId u8 (each array whole, res^2 entries), then
// per exit a u32 length and its name | FNV-1a 64 of the payload
namespace {

struct NavCacheReader {
    std::FILE* f = nullptr;
    uint64_t hash = 0xcbf29ce484222325ull;
    bool ok = true;
    explicit NavCacheReader(const char* path) : f(std::fopen(path, "rb")) { ok = f != nullptr; }
    ~NavCacheReader() { if (f) std::fclose(f); }
    bool read(void* dst, size_t bytes, bool hashed = true) {
        if (!ok) return false;
        if (std::fread(dst, 1, bytes, f) != bytes) return ok = false;
        if (hashed) {
            const unsigned char* b = static_cast<const unsigned char*>(dst);
            for (size_t i = 0; i < bytes; ++i) { hash ^= b[i]; hash *= 0x100000001b3ull; }
        }
        return true;
    }
};

constexpr char NAV_MAGIC[8] = {'S', 'W', 'N', 'A', 'V', 'F', '0', '1'};
constexpr uint32_t NAV_VERSION = 2;     // nav::VERSION (include/swarm/nav_field.hpp:60)
constexpr int NAV_FIT_CLASS = 0;        // nav::FIT

}  // namespace

extern "C" int swarm_nav_cache_read(const char* path, uint64_t expected_key, SwarmNavCell* cells, int64_t capacity,
                                    int32_t* res_out, float* origin, float* cell, float* inv_cell) {
    if (!path || !res_out || !origin || !cell || !inv_cell) return SWARM_E_INVALID;
    NavCacheReader in(path);
    char magic[8];
    if (!in.read(magic, 8, false) || std::memcmp(magic, NAV_MAGIC, 8) != 0) return SWARM_E_INVALID;
    uint32_t version = 0, res = 0, exits = 0;
    uint64_t key = 0;
    float o = 0.0f, c = 0.0f, ic = 0.0f;
    if (!in.read(&version, 4) || !in.read(&res, 4) || !in.read(&o, 4) || !in.read(&c, 4) || !in.read(&ic, 4) ||
        !in.read(&exits, 4) || !in.read(&key, 8))
        return SWARM_E_INVALID;
    if (version != NAV_VERSION || res == 0 || res > 100000 || exits > 255) return SWARM_E_INVALID;
    if (expected_key != 0 && key != expected_key) return SWARM_E_INVALID;
    *res_out = int32_t(res);
    *origin = o;
    *cell = c;
    *inv_cell = ic;
    const size_t n = size_t(res) * size_t(res);
    if (!cells) return SWARM_OK;   // a size query
    if (capacity < int64_t(n)) return SWARM_E_INVALID;
    std::vector<float> floorZ(n), dist(n);
    std::vector<uint8_t> cls(n), out(n), exitId(n);
    std::vector<int8_t> region(n);
    std::vector<int32_t> anchor(n);
    if (!in.read(floorZ.data(), n * 4) || !in.read(cls.data(), n) || !in.read(out.data(), n) || !in.read(region.data(), n) ||
        !in.read(dist.data(), n * 4) || !in.read(anchor.data(), n * 4) || !in.read(exitId.data(), n))
        return SWARM_E_INVALID;
    for (uint32_t e = 0; e < exits; ++e) {
        uint32_t len = 0;
        if (!in.read(&len, 4) || len > 1000) return SWARM_E_INVALID;
        std::vector<char> name(len);
        if (len && !in.read(name.data(), len)) return SWARM_E_INVALID;
    }
    uint64_t sum = 0;
    if (!in.read(&sum, 8, false) || sum != in.hash) return SWARM_E_INVALID;
    char extra;
    if (std::fread(&extra, 1, 1, in.f) != 0) return SWARM_E_INVALID;   // nothing after the checksum
    // nav::gpuCells (src/nav_field.cpp:443-454): the anchor's centre (nav::Grid::centre, src/nav_field.cpp:32-35:
    // double arithmetic, rounded once; an unreachable cell's own centre), the distance, the info bits
    const double cd = double(c);
    for (size_t i = 0; i < n; ++i) {
        const int a = anchor[i] >= 0 ? int(anchor[i]) : int(i);
        if (size_t(a) >= n) return SWARM_E_INVALID;
        SwarmNavCell& g = cells[i];
        g.anchor_x = float(double(o) + (double(a % int(res)) + 0.5) * cd);
        g.anchor_y = float(double(o) + (double(a / int(res)) + 0.5) * cd);
        g.dist = dist[i];
        g.info = uint32_t(exitId[i]) | (cls[i] == NAV_FIT_CLASS ? SWARM_NAV_FIT : 0u) | (std::isfinite(dist[i]) ? SWARM_NAV_REACHABLE : 0u);
    }
    return SWARM_OK;
}

namespace {
constexpr char CHOICE_MAGIC[8] = {'S', 'W', 'C', 'H', 'O', 'I', '0', '1'};
constexpr uint32_t CHOICE_VERSION = 6;   // nav::CHOICE_VERSION (include/swarm/exit_choice.hpp:121)
constexpr uint32_t CHOICE_K = 24;        // nav::CHOICE_K
}  // namespace

// nav::loadChoice (src/exit_choice.cpp:399-427): the header, then index and entries straight into the caller's
// buffers, the exits' widths and names, the checksum; nothing may follow it
extern "C" int swarm_choice_cache_read(const char* path, uint64_t expected_key, uint32_t* index, int64_t index_capacity,
                                       SwarmNavChoiceCell* entries, int64_t entry_capacity, double* width_m, int32_t* res_out,
                                       float* origin, float* cell, float* inv_cell, int32_t* n_exits, int64_t* n_entries) {
    if (!path || !res_out || !origin || !cell || !inv_cell || !n_exits || !n_entries) return SWARM_E_INVALID;
    if ((index == nullptr) != (entries == nullptr)) return SWARM_E_INVALID;
    NavCacheReader in(path);
    char magic[8];
    if (!in.read(magic, 8, false) || std::memcmp(magic, CHOICE_MAGIC, 8) != 0) return SWARM_E_INVALID;
    uint32_t version = 0, k = 0, res = 0, exits = 0;
    uint64_t key = 0, ne = 0;
    float o = 0.0f, c = 0.0f, ic = 0.0f;
    if (!in.read(&version, 4) || !in.read(&k, 4) || !in.read(&res, 4) || !in.read(&o, 4) || !in.read(&c, 4) ||
        !in.read(&ic, 4) || !in.read(&exits, 4) || !in.read(&key, 8))
        return SWARM_E_INVALID;
    if (version != CHOICE_VERSION || k != CHOICE_K || res == 0 || res > 100000 || exits > SWARM_CHOICE_MAX_EXITS)
        return SWARM_E_INVALID;
    if (expected_key != 0 && key != expected_key) return SWARM_E_INVALID;
    const size_t cells = size_t(res) * size_t(res);
    if (!in.read(&ne, 8) || ne > cells) return SWARM_E_INVALID;
    *res_out = int32_t(res);
    *origin = o;
    *cell = c;
    *inv_cell = ic;
    *n_exits = int32_t(exits);
    *n_entries = int64_t(ne);
    if (!index) return SWARM_OK;   // a size query: the header alone
    if (index_capacity < int64_t(cells) || entry_capacity < int64_t(ne)) return SWARM_E_INVALID;
    if (!in.read(index, cells * 4) || !in.read(entries, size_t(ne) * sizeof(SwarmNavChoiceCell))) return SWARM_E_INVALID;
    for (uint32_t e = 0; e < exits; ++e) {
        double w = 0.0;
        uint32_t len = 0;
        if (!in.read(&w, 8) || !in.read(&len, 4) || len > 1000) return SWARM_E_INVALID;
        std::vector<char> name(len);
        if (len && !in.read(name.data(), len)) return SWARM_E_INVALID;
        if (width_m) width_m[e] = w;
    }
    uint64_t sum = 0;
    if (!in.read(&sum, 8, false) || sum != in.hash) return SWARM_E_INVALID;
    char extra;
    if (std::fread(&extra, 1, 1, in.f) != 0) return SWARM_E_INVALID;   // nothing after the checksum
    for (size_t i = 0; i < cells; ++i)
        if ((index[i] & SWARM_CHOICE_INDEX_MASK) > ne) return SWARM_E_INVALID;   // an entry the file does not hold
    return SWARM_OK;
}
