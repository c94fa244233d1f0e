// Oracle (test infrastructure only): resolves to the component-framework stand-in.
#pragma once
#include "component.h"
