// Empty stand-in: the reference's accelerator sources include this glm header
// but use nothing from it.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "../glm.hpp"
