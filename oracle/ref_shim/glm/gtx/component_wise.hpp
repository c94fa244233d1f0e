// Oracle (test infrastructure only): glm sub-header stand-in; everything lives in glm.hpp.
#pragma once
#include "../glm.hpp"
