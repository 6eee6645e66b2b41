/* The CUDA-samples timer calls the reference's CUDA build makes (src/Replica.cpp,
 * src/Simulation.cpp; only under its timing switch), as no-ops.  TEST INFRASTRUCTURE
 * ONLY: for linking the reference's own call sites against the drop-in library. */
#pragma once

class StopWatchInterface {
};

inline bool sdkCreateTimer(StopWatchInterface **t)
{
    *t = new StopWatchInterface();
    return true;
}
inline bool sdkDeleteTimer(StopWatchInterface **t)
{
    delete *t;
    *t = nullptr;
    return true;
}
inline bool sdkStartTimer(StopWatchInterface **) { return true; }
inline bool sdkStopTimer(StopWatchInterface **) { return true; }
inline float sdkGetTimerValue(StopWatchInterface **) { return 0.0f; }
inline float sdkGetAverageTimerValue(StopWatchInterface **) { return 0.0f; }
