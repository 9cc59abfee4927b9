// glm subset for the host-compiled reference oracle; everything lives in glm.hpp.
#pragma once
#include "../glm.hpp"
