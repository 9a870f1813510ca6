// Stand-in for the reference's sdf.h: the payload type named by TriangleBvh's interface.
#pragma once
#include <neural-graphics-primitives/common.h>
#include <tiny-cuda-nn/gpu_memory.h>
NGP_NAMESPACE_BEGIN
struct SdfPayload { Eigen::Vector3f dir; uint32_t idx; uint16_t n_steps; bool alive; };
NGP_NAMESPACE_END
