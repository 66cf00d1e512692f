// genie/utility/Timing.h -- wall-clock helpers of the legacy interface
// (reference src/genie/utility/Timing.h:22-37).
#ifndef GENIE_UTILITY_TIMING_H_
#define GENIE_UTILITY_TIMING_H_

typedef unsigned long long u64;

// Microseconds on a monotonic clock.
unsigned long long getTime();
// Milliseconds between two getTime() readings.
double getInterval(unsigned long long start, unsigned long long stop);

#endif
