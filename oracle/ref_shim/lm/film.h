// Oracle (test infrastructure only): the reference's camera source includes the film header but
// uses nothing from it; this file stands in for it.
#pragma once
#include <lm/core.h>
