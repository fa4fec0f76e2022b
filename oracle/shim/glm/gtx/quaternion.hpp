// Oracle test infrastructure: forwards to the project's glm-compatible header.
#pragma once
#include "../glm.hpp"
