// glm::pi for the reference's sources; defined with the rest of the minimal
// vector-math header.
#pragma once
#include "../glm.hpp"
