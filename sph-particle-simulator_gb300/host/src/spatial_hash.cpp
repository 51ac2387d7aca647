// Host SpatialHash over the GPU grid ABI (sphx_grid_*): the reference's class and
// semantics (src/spatial_hash.h, src/spatial_hash.cpp), with build and queries on the GPU.
#include "spatial_hash.h"

#include <cmath>
#include <stdexcept>
#include <string>

#include "sphx.h"

namespace sph {

namespace {
void check(int rc, const char* where) {
    if (rc != SPHX_OK) throw std::runtime_error(std::string(where) + ": " + sphx_strerror(rc));
}
}  // namespace

SpatialHash::SpatialHash(float cell_size)
    : cell_size_(cell_size), inv_cell_size_(1.0f / cell_size) {}

SpatialHash::~SpatialHash() { sphx_grid_destroy(grid_); }

void SpatialHash::ensure_grid(size_t n) const {
    if (grid_ && grid_capacity_ >= n) return;
    sphx_grid_destroy(grid_);
    grid_ = nullptr;
    size_t cap = grid_capacity_ ? grid_capacity_ : 1024;
    while (cap < n) cap *= 2;
    check(sphx_grid_create(&grid_, cap), "sphx_grid_create");
    grid_capacity_ = cap;
}

// SpatialHash::build (src/spatial_hash.cpp:15-25)
void SpatialHash::build(const std::vector<glm::vec3>& positions) {
    clear();
    ensure_grid(positions.size());
    std::vector<float> xyz(3 * positions.size());
    for (size_t i = 0; i < positions.size(); ++i) {
        xyz[3 * i] = positions[i].x;
        xyz[3 * i + 1] = positions[i].y;
        xyz[3 * i + 2] = positions[i].z;
    }
    check(sphx_grid_build(grid_, positions.size(), xyz.data(), cell_size_), "sphx_grid_build");
    n_ = positions.size();
    built_ = true;
}

// SpatialHash::query (src/spatial_hash.cpp:27-29)
std::vector<size_t> SpatialHash::query(const glm::vec3& position, float radius) const {
    return query_squared(position, radius * radius);
}

std::vector<size_t> SpatialHash::query_squared(const glm::vec3& position,
                                               float radius_squared) const {
    std::vector<size_t> counts, idx;
    query_squared_batch(std::vector<glm::vec3>{position}, radius_squared, counts, idx);
    return idx;
}

void SpatialHash::query_squared_batch(const std::vector<glm::vec3>& positions,
                                      float radius_squared, std::vector<size_t>& counts,
                                      std::vector<size_t>& indices) const {
    const size_t nq = positions.size();
    counts.assign(nq, 0);
    indices.clear();
    if (!built_ || n_ == 0 || nq == 0) return;
    std::vector<float> q(3 * nq);
    for (size_t i = 0; i < nq; ++i) {
        q[3 * i] = positions[i].x;
        q[3 * i + 1] = positions[i].y;
        q[3 * i + 2] = positions[i].z;
    }
    std::vector<int64_t> c(nq);
    size_t total = 0;
    check(sphx_grid_query(grid_, nq, q.data(), radius_squared, c.data(), nullptr, &total),
          "sphx_grid_query");
    std::vector<int64_t> idx(total ? total : 1);
    size_t total2 = total;
    check(sphx_grid_query(grid_, nq, q.data(), radius_squared, c.data(), idx.data(), &total2),
          "sphx_grid_query");
    for (size_t i = 0; i < nq; ++i) counts[i] = static_cast<size_t>(c[i]);
    indices.assign(idx.begin(), idx.begin() + static_cast<std::ptrdiff_t>(total2));
}

// get_cell_particles (src/spatial_hash.cpp:59-63): nullptr for an empty cell
const std::vector<size_t>* SpatialHash::get_cell_particles(int x, int y, int z) const {
    if (!built_ || n_ == 0) return nullptr;
    const uint64_t key = (static_cast<uint64_t>(x & 0x1FFFFF) << 42) |
                         (static_cast<uint64_t>(y & 0x1FFFFF) << 21) |
                         static_cast<uint64_t>(z & 0x1FFFFF);
    auto it = cell_cache_.find(key);
    if (it != cell_cache_.end()) return &it->second;
    size_t cnt = 0;
    check(sphx_grid_cell(grid_, x, y, z, nullptr, &cnt), "sphx_grid_cell");
    if (cnt == 0) return nullptr;
    std::vector<int64_t> ids(cnt);
    size_t cnt2 = cnt;
    check(sphx_grid_cell(grid_, x, y, z, ids.data(), &cnt2), "sphx_grid_cell");
    std::vector<size_t>& v = cell_cache_[key];
    v.assign(ids.begin(), ids.begin() + static_cast<std::ptrdiff_t>(cnt2));
    return &v;
}

void SpatialHash::clear() {
    built_ = false;
    n_ = 0;
    cell_cache_.clear();
}

size_t SpatialHash::get_total_cells() const {
    if (!built_) return 0;
    size_t cells = 0, mx = 0;
    check(sphx_grid_info(grid_, &cells, &mx), "sphx_grid_info");
    return cells;
}

size_t SpatialHash::get_max_particles_per_cell() const {
    if (!built_) return 0;
    size_t cells = 0, mx = 0;
    check(sphx_grid_info(grid_, &cells, &mx), "sphx_grid_info");
    return mx;
}

namespace spatial_hash_utils {

float estimate_cell_size(float smoothing_length) { return smoothing_length; }

std::vector<uint64_t> precompute_hashes(const std::vector<glm::vec3>& positions,
                                        float inv_cell_size) {
    std::vector<uint64_t> out;
    out.reserve(positions.size());
    for (const glm::vec3& p : positions) {
        const int x = static_cast<int>(std::floor(p.x * inv_cell_size));
        const int y = static_cast<int>(std::floor(p.y * inv_cell_size));
        const int z = static_cast<int>(std::floor(p.z * inv_cell_size));
        out.push_back((static_cast<uint64_t>(x & 0x1FFFFF) << 42) |
                      (static_cast<uint64_t>(y & 0x1FFFFF) << 21) |
                      static_cast<uint64_t>(z & 0x1FFFFF));
    }
    return out;
}

}  // namespace spatial_hash_utils

}  // namespace sph
