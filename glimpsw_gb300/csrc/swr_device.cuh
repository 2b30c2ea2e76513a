// The device helpers live in the public header (user shaders compiled against include/swr/ use them).
#pragma once
#include "../../include/swr/device.cuh"
