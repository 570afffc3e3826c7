// glm/gtx/normal.hpp: triangleNormal is in glm.hpp (test infrastructure).
#include "../glm.hpp"
