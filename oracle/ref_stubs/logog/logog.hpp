/* The logging macros the reference uses (src/*.cpp), as no-ops, for building its MC
 * layer as a checker.  TEST INFRASTRUCTURE ONLY. */
#pragma once

#define LOGOG_DEBUG(...) ((void)0)
#define LOGOG_INFO(...) ((void)0)
#define LOGOG_WARN(...) ((void)0)
#define LOGOG_ERROR(...) ((void)0)
#define LOGOG_INITIALIZE() ((void)0)
#define LOGOG_SHUTDOWN() ((void)0)
#define LOGOG_SET_LEVEL(x) ((void)0)
#define LOGOG_LEVEL_ALL 0
#define LOGOG_LEVEL_ERROR 0
#define LOGOG_LEVEL_INFO 0
#define LOGOG_LEVEL_NONE 0
#define LOGOG_LEVEL_WARN 0
#define LOGOG_USE_PREFIX 0

namespace logog {
struct Cout {
};
}  // namespace logog
