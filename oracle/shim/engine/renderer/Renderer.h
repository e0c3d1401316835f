// Stand-in for src/engine/renderer/Renderer.h: the marcher reads only the
// swapchain extent (RayMarcher.cpp:86-89).  Oracle build only.
#pragma once
#include <cstdint>

struct FmShimExtent { uint32_t width = 0, height = 0; };
struct FmShimVulkan { FmShimExtent SwapchainExtent; };
extern FmShimVulkan Vulkan;
