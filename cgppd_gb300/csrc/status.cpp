// status.cpp -- per-thread last-error record (see status.h).
#include "status.h"

#include <cstdio>
#include <cstring>

namespace {
thread_local int t_code = 0;
thread_local char t_msg[512] = {0};
}  // namespace

int cgppd_check(cudaError_t err, const char *where)
{
    if (err == cudaSuccess)
        return 0;
    t_code = (int)err;
    std::snprintf(t_msg, sizeof(t_msg), "%s: CUDA error %d (%s)", where, (int)err, cudaGetErrorString(err));
    std::fprintf(stderr, "cgppd: %s\n", t_msg);
    return -1;
}

int cgppd_fail(const char *msg)
{
    t_code = -1;
    std::snprintf(t_msg, sizeof(t_msg), "%s", msg);
    std::fprintf(stderr, "cgppd: %s\n", t_msg);
    return -1;
}

extern "C" int cgppd_get_last_error(char *buf, int buflen)
{
    int code = t_code;
    if (buf != nullptr && buflen > 0) {
        std::strncpy(buf, t_msg, (size_t)buflen - 1);
        buf[buflen - 1] = 0;
    }
    t_code = 0;
    t_msg[0] = 0;
    return code;
}
