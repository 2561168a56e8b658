// Stand-in for the reference's src/core/Buffer.h (an OpenGL buffer wrapper,
// which needs glad and GLFW).  src/accelerator/BVH.h includes it but BVH.cpp
// uses nothing from it.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>
