// Smoothing kernels of the drop-in API (reference semantics: src/kernels.cpp:11-236,
// 292-296).  Every expression keeps the reference's float operation order (the library
// is built with -ffp-contract=off), so W / gradW / laplacianW return the reference's bits.
#include "kernels.h"

#include <cmath>
#include <stdexcept>

namespace sph {

namespace {

constexpr float kPi = static_cast<float>(M_PI);

// The cubic-spline piecewise polynomial in q for a normalisation sigma
// (W_1d / W_2d / W_3d, kernels.cpp:38-66)
float cubic_value(float sigma, float q) {
    if (q >= 0.0f && q <= 1.0f) return sigma * (2.0f / 3.0f - q * q + 0.5f * q * q * q);
    if (q > 1.0f && q <= 2.0f) {
        const float t = 2.0f - q;
        return sigma * (1.0f / 6.0f * t * t * t);
    }
    return 0.0f;
}

// gradW_1d / _2d / _3d (kernels.cpp:68-108): dW/dq along r / |r|, then / h
glm::vec3 cubic_gradient(float sigma, float h, const glm::vec3& r, float q) {
    const float r_len = glm::length(r);
    if (r_len < 1e-6f) return glm::vec3(0.0f);
    glm::vec3 g(0.0f);
    if (q >= 0.0f && q <= 1.0f) {
        g = sigma * (-2.0f * q + 1.5f * q * q) * (r / r_len);
    } else if (q > 1.0f && q <= 2.0f) {
        const float t = 2.0f - q;
        g = -sigma * (0.5f * t * t) * (r / r_len);
    }
    return g / h;
}

// laplacianW_1d / _2d / _3d (kernels.cpp:110-138)
float cubic_laplacian(float sigma, float h_sq, float q) {
    if (q >= 0.0f && q <= 1.0f) return sigma * (-2.0f + 3.0f * q) / h_sq;
    if (q > 1.0f && q <= 2.0f) return sigma * (2.0f - q) / h_sq;
    return 0.0f;
}

}  // namespace

Kernel::Kernel(float h) : h_(h), h_inv_(1.0f / h), h_sq_(h * h), norm_(0.0f) {}

// Only h and its derived values change; normalisations keep their construction-time
// values, as in the reference (kernels.cpp:16-20).
void Kernel::set_smoothing_length(float h) {
    h_ = h;
    h_inv_ = 1.0f / h;
    h_sq_ = h * h;
}

CubicSplineKernel::CubicSplineKernel(float h) : Kernel(h) {
    sigma_3d_ = 1.0f / (kPi * h * h * h);
    sigma_2d_ = 10.0f / (7.0f * kPi * h * h);
    sigma_1d_ = 2.0f / (3.0f * h);
    norm_ = sigma_3d_;
}

float CubicSplineKernel::W_1d(float q) const { return cubic_value(sigma_1d_, q); }
float CubicSplineKernel::W_2d(float q) const { return cubic_value(sigma_2d_, q); }
float CubicSplineKernel::W_3d(float q) const { return cubic_value(sigma_3d_, q); }

glm::vec3 CubicSplineKernel::gradW_1d(const glm::vec3& r, float q) const {
    return cubic_gradient(sigma_1d_, h_, r, q);
}
glm::vec3 CubicSplineKernel::gradW_2d(const glm::vec3& r, float q) const {
    return cubic_gradient(sigma_2d_, h_, r, q);
}
glm::vec3 CubicSplineKernel::gradW_3d(const glm::vec3& r, float q) const {
    return cubic_gradient(sigma_3d_, h_, r, q);
}

float CubicSplineKernel::laplacianW_1d(float q) const { return cubic_laplacian(sigma_1d_, h_sq_, q); }
float CubicSplineKernel::laplacianW_2d(float q) const { return cubic_laplacian(sigma_2d_, h_sq_, q); }
float CubicSplineKernel::laplacianW_3d(float q) const { return cubic_laplacian(sigma_3d_, h_sq_, q); }

float CubicSplineKernel::W(const glm::vec3& r) const {
    return W_3d(kernel_utils::compute_q(r, h_));
}
glm::vec3 CubicSplineKernel::gradW(const glm::vec3& r) const {
    return gradW_3d(r, kernel_utils::compute_q(r, h_));
}
float CubicSplineKernel::laplacianW(const glm::vec3& r) const {
    return laplacianW_3d(kernel_utils::compute_q(r, h_));
}
float CubicSplineKernel::W_2D(const glm::vec2& r) const { return W_2d(glm::length(r) / h_); }
float CubicSplineKernel::W_1D(float r) const { return W_1d(std::abs(r) / h_); }

WendlandC2Kernel::WendlandC2Kernel(float h) : Kernel(h) {
    norm_factor_ = 21.0f / (2.0f * kPi * h * h * h);
}

// norm (1 - q/2)^4 (2q + 1) for q < 2
float WendlandC2Kernel::W(const glm::vec3& r) const {
    const float q = kernel_utils::compute_q(r, h_);
    if (q >= 2.0f) return 0.0f;
    const float t = 1.0f - 0.5f * q;
    return norm_factor_ * t * t * t * t * (2.0f * q + 1.0f);
}

// norm dW/dq r / (|r| h), dW/dq = -5 (1 - q/2)^3 q
glm::vec3 WendlandC2Kernel::gradW(const glm::vec3& r) const {
    const float r_len = glm::length(r);
    if (r_len < 1e-6f) return glm::vec3(0.0f);
    const float q = r_len / h_;
    if (q >= 2.0f) return glm::vec3(0.0f);
    const float t = 1.0f - 0.5f * q;
    const float dw_dq = -5.0f * t * t * t * q;
    return norm_factor_ * dw_dq * (r / (r_len * h_));
}

float WendlandC2Kernel::laplacianW(const glm::vec3& r) const {
    const float q = kernel_utils::compute_q(r, h_);
    if (q >= 2.0f) return 0.0f;
    const float t = 1.0f - 0.5f * q;
    return norm_factor_ * (5.0f / h_sq_) * t * t * (5.0f * q - 3.0f);
}

GaussianKernel::GaussianKernel(float h) : Kernel(h) {
    sigma_sq_inv_ = 1.0f / (h * h);
    norm_ = 1.0f / std::pow(kPi * h * h, 1.5f);
}

float GaussianKernel::W(const glm::vec3& r) const {
    const float r_sq = glm::dot(r, r);
    return norm_ * std::exp(-r_sq * sigma_sq_inv_);
}

glm::vec3 GaussianKernel::gradW(const glm::vec3& r) const {
    const float r_sq = glm::dot(r, r);
    const float e = std::exp(-r_sq * sigma_sq_inv_);
    return -2.0f * sigma_sq_inv_ * norm_ * e * r;
}

float GaussianKernel::laplacianW(const glm::vec3& r) const {
    const float r_sq = glm::dot(r, r);
    const float e = std::exp(-r_sq * sigma_sq_inv_);
    return 2.0f * sigma_sq_inv_ * norm_ * e * (2.0f * sigma_sq_inv_ * r_sq - 3.0f);
}

std::unique_ptr<Kernel> create_kernel(KernelType type, float smoothing_length) {
    switch (type) {
        case KernelType::CUBIC_SPLINE:
            return std::make_unique<CubicSplineKernel>(smoothing_length);
        case KernelType::WENDLAND_C2:
            return std::make_unique<WendlandC2Kernel>(smoothing_length);
        case KernelType::GAUSSIAN:
            return std::make_unique<GaussianKernel>(smoothing_length);
    }
    throw std::invalid_argument("Unknown kernel type");
}

namespace kernel_utils {

float estimate_smoothing_length(float particle_spacing, float neighbor_count) {
    return particle_spacing * std::pow(neighbor_count / 50.0f, 1.0f / 3.0f);
}

}  // namespace kernel_utils

}  // namespace sph
