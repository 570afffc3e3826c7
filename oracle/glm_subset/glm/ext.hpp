// glm/ext.hpp: the GLM subset lives in glm.hpp (test infrastructure).
#include "glm.hpp"
