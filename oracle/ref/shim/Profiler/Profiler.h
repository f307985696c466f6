// Stand-in for the engine's Profiler/Profiler.h: the profiler is compiled out
// in the reference too (ACTIVATE_PROFILER 0). Reference-build recipe only.
#pragma once
#define PROFILE_FUNC()
#define PROFILE_SCOPE(name)
