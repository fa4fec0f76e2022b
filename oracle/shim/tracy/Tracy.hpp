// Oracle test infrastructure: Tracy profiler macros compiled out. The reference fetches
// Tracy over the network at configure time; the oracle build only needs the macros to
// expand to nothing.
#pragma once
#define ZoneScoped
#define ZoneScopedN(name)
#define ZoneScopedC(color)
#define ZoneScopedNC(name, color)
#define FrameMark
#define FrameMarkNamed(name)
#define TracyAlloc(ptr, size)
#define TracyFree(ptr)
