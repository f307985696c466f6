// Stand-in for the engine's TransformSystem.h: only the `Changed` tag and the
// glm headers it pulls in. Reference-build recipe only (test infrastructure).
#pragma once
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>
struct Changed {};
