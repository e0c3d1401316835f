// Stand-in for src/engine/utils/PerformanceTimer.h: profiling scopes compile
// to nothing in the oracle build.
#pragma once
#define PROFILE_SCOPE(name)
#define PROFILE_FUNCTION()
