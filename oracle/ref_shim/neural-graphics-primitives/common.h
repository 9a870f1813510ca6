// Stand-in for the reference's common.h (which pulls in the GUI/logging stack): only the
// macros, aliases and the sign() helper that the hot-path headers use.  Test infrastructure.
#pragma once
#include <Eigen/Dense>
#include <cmath>
#include <cstdint>
#include <functional>

#define NGP_NAMESPACE_BEGIN namespace ngp {
#define NGP_NAMESPACE_END }
#define NGP_HOST_DEVICE
#define NGP_PRAGMA_UNROLL
#define NGP_PRAGMA_NO_UNROLL

NGP_NAMESPACE_BEGIN
using Vector2i32 = Eigen::Matrix<uint32_t, 2, 1>;
using Vector4i32 = Eigen::Matrix<uint32_t, 4, 1>;
enum class EMeshSdfMode : int { Watertight, Raystab, PathEscape };
// sign(x) = copysignf(1, x), as the reference defines it
inline float sign(float x) { return copysignf(1.0, x); }
NGP_NAMESPACE_END
