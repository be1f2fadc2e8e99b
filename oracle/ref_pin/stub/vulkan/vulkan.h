/* Stand-in for the Vulkan SDK header that vulkan_acceleration_structure_util.h
 * includes.  The decoders use no Vulkan declarations: they need only
 * <cstdint>, <cmath> and CUDA's float3 / float4 (vector_types.h), which the
 * pin harness includes first. */
#pragma once
