// Smoothing-kernel API of the GB300 drop-in engine.
//
// Same namespace, class names, member functions and semantics as the reference's
// kernels.h (src/kernels.h:8-132): the abstract Kernel, CubicSplineKernel,
// WendlandC2Kernel, GaussianKernel, KernelType and create_kernel, and kernel_utils.  These
// are scalar host evaluations for user code (the reference's equations:: call them once
// per pair); SPHEngine::step never calls them -- its per-pair kernels run on the GPU with
// the same float operations (select one with SPHEngine::set_kernel_type).
//
// Differences from the reference, all deliberate:
//  * The AVX2 helpers of kernels.h:103-113 are not provided (x86-only, and the reference's
//    gradient helper returns the kernel value, kernels.cpp:279-283).
//  * create_kernel's unknown-type error is the reference's: std::invalid_argument.
#pragma once

#include <glm/glm.hpp>
#include <memory>
#include <vector>

namespace sph {

// Smoothing kernel base class (src/kernels.h:9-32).
class Kernel {
   protected:
    float h_;      // smoothing length
    float h_inv_;  // 1/h
    float h_sq_;   // h^2
    float norm_;   // normalisation constant

   public:
    explicit Kernel(float h);
    virtual ~Kernel() = default;

    virtual float W(const glm::vec3& r) const = 0;
    virtual glm::vec3 gradW(const glm::vec3& r) const = 0;
    virtual float laplacianW(const glm::vec3& r) const = 0;

    float get_smoothing_length() const { return h_; }
    void set_smoothing_length(float h);

    float get_support_radius() const { return 2.0f * h_; }
    float get_cutoff_radius() const { return get_support_radius(); }
};

// Cubic spline kernel (src/kernels.h:35-65, kernels.cpp:23-163).
class CubicSplineKernel : public Kernel {
   private:
    float sigma_1d_;
    float sigma_2d_;
    float sigma_3d_;

    float W_1d(float q) const;
    float W_2d(float q) const;
    float W_3d(float q) const;

    glm::vec3 gradW_1d(const glm::vec3& r, float q) const;
    glm::vec3 gradW_2d(const glm::vec3& r, float q) const;
    glm::vec3 gradW_3d(const glm::vec3& r, float q) const;

    float laplacianW_1d(float q) const;
    float laplacianW_2d(float q) const;
    float laplacianW_3d(float q) const;

   public:
    explicit CubicSplineKernel(float h);

    float W(const glm::vec3& r) const override;
    glm::vec3 gradW(const glm::vec3& r) const override;
    float laplacianW(const glm::vec3& r) const override;

    float W_3D(const glm::vec3& r) const { return W(r); }
    float W_2D(const glm::vec2& r) const;
    float W_1D(float r) const;
};

// Wendland C2 kernel (src/kernels.h:68-78, kernels.cpp:166-200).
class WendlandC2Kernel : public Kernel {
   private:
    float norm_factor_;

   public:
    explicit WendlandC2Kernel(float h);

    float W(const glm::vec3& r) const override;
    glm::vec3 gradW(const glm::vec3& r) const override;
    float laplacianW(const glm::vec3& r) const override;
};

// Gaussian kernel (src/kernels.h:81-91, kernels.cpp:203-225).
class GaussianKernel : public Kernel {
   private:
    float sigma_sq_inv_;

   public:
    explicit GaussianKernel(float h);

    float W(const glm::vec3& r) const override;
    glm::vec3 gradW(const glm::vec3& r) const override;
    float laplacianW(const glm::vec3& r) const override;
};

// Kernel factory (src/kernels.h:94-100, kernels.cpp:226-236); the numbering is also the
// sphx C ABI's SPHX_KERNEL_*.
enum class KernelType { CUBIC_SPLINE, WENDLAND_C2, GAUSSIAN };

std::unique_ptr<Kernel> create_kernel(KernelType type, float smoothing_length);

namespace kernel_utils {

// q = |r| / h (src/kernels.h:117-119)
inline float compute_q(const glm::vec3& r, float h) { return glm::length(r) / h; }

// |r|^2 <= (support_factor h)^2 (src/kernels.h:122-124)
inline bool within_support(const glm::vec3& r, float h, float support_factor = 2.0f) {
    return glm::dot(r, r) <= (support_factor * h) * (support_factor * h);
}

// h from the particle spacing and a target neighbour count (src/kernels.cpp:292-296)
float estimate_smoothing_length(float particle_spacing, float neighbor_count = 50.0f);

}  // namespace kernel_utils

}  // namespace sph
