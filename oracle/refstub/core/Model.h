// Stand-in for the reference's src/core/Model.h (assimp and OpenGL model
// classes).  src/accelerator/BVH.h includes it but BVH.cpp uses nothing from
// it.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <glm/glm.hpp>
