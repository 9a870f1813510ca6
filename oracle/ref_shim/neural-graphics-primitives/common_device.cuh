// Stand-in for the reference's common_device.cuh: the hot-path headers need nothing from it
// beyond common.h and the tiny-cuda-nn helpers.  Test infrastructure.
#pragma once
#include <neural-graphics-primitives/common.h>
#include <tiny-cuda-nn/common.h>
