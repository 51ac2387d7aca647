// GPU-backed drop-in for the reference's SpatialHash (src/spatial_hash.h:12-88).
//
// build() sorts the positions into cells of cell_size on the GPU (the same cells as the
// reference: floor(x / cell) with inv = 1.0f / cell_size); query()/query_squared() return
// exactly the reference's lists -- every particle with dot(x - p, x - p) <= r^2, in the
// reference's order (stencil cells lexicographic, then insertion order) -- computed on
// the GPU through the sphx C ABI.  Positions with a NaN/inf coordinate belong to no cell
// here (the reference files them under an implementation-defined cell); lists are
// unaffected because no distance test with them passes.
#pragma once

#include <glm/glm.hpp>
#include <cstdint>
#include <memory>
#include <unordered_map>
#include <vector>

struct sphx_grid;

namespace sph {

class SpatialHash {
   public:
    explicit SpatialHash(float cell_size = 0.02f);
    ~SpatialHash();
    SpatialHash(const SpatialHash&) = delete;
    SpatialHash& operator=(const SpatialHash&) = delete;

    void build(const std::vector<glm::vec3>& positions);
    std::vector<size_t> query(const glm::vec3& position, float radius) const;
    std::vector<size_t> query_squared(const glm::vec3& position, float radius_squared) const;
    // Many queries in one GPU launch (lists concatenated; counts[i] per query).
    void query_squared_batch(const std::vector<glm::vec3>& positions, float radius_squared,
                             std::vector<size_t>& counts, std::vector<size_t>& indices) const;
    const std::vector<size_t>* get_cell_particles(int x, int y, int z) const;
    void clear();
    size_t get_total_cells() const;
    size_t get_max_particles_per_cell() const;
    float get_cell_size() const { return cell_size_; }
    void set_cell_size(float cell_size) {
        cell_size_ = cell_size;
        inv_cell_size_ = 1.0f / cell_size_;
    }

   private:
    void ensure_grid(size_t n) const;
    float cell_size_;
    float inv_cell_size_;
    mutable sphx_grid* grid_ = nullptr;
    mutable size_t grid_capacity_ = 0;
    size_t n_ = 0;
    bool built_ = false;
    mutable std::unordered_map<uint64_t, std::vector<size_t>> cell_cache_;
};

namespace spatial_hash_utils {
// Cell size estimate (src/spatial_hash.cpp:183-187): the smoothing length.
float estimate_cell_size(float smoothing_length);
// 64-bit keys with 21 bits per cell coordinate (src/spatial_hash.h:20-27).
std::vector<uint64_t> precompute_hashes(const std::vector<glm::vec3>& positions,
                                        float inv_cell_size);
}  // namespace spatial_hash_utils

}  // namespace sph
