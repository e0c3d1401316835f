// Stand-in for the reference's precompiled header (src/engine/hzpch.h).
// Keeps the STL, spdlog, glm (with the same three GLM_FORCE_* switches as the
// reference, hzpch.h:22-24) and Eigen; drops Vulkan, GLFW, yaml-cpp and ImGui,
// which the marcher translation units do not use.  Oracle build only.
#pragma once

#include <algorithm>
#include <array>
#include <atomic>
#include <barrier>
#include <cassert>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <filesystem>
#include <functional>
#include <iostream>
#include <list>
#include <memory>
#include <mutex>
#include <optional>
#include <queue>
#include <string>
#include <thread>
#include <vector>

#include <spdlog/spdlog.h>

#define GLM_FORCE_RADIANS
#define GLM_FORCE_DEPTH_ZERO_TO_ONE
#define GLM_FORCE_LEFT_HANDED

#include <glm/glm.hpp>
#include <glm/vec4.hpp>
#include <glm/mat4x4.hpp>
#include <glm/gtc/quaternion.hpp>
#include <glm/ext/matrix_transform.hpp>
#include <glm/ext/matrix_clip_space.hpp>

#include <Eigen/Dense>

#define HZ_ASSERT(x, ...) { if (!(x)) { SPDLOG_ERROR(__VA_ARGS__); assert(false); } }
