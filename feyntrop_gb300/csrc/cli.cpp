// `feyntrop` command: the reference's CLI contract (srcs/feyntrop.cpp:20-281) on the
// GPU.  stdin: the JSON input; stdout: the JSON result; stderr: diagnostics.  Any
// error prints its message on stderr and exits non-zero, as the reference's
// uncaught exceptions do.
#include <cstdio>
#include <iostream>
#include <iterator>
#include <string>

#include "../../include/feyntrop_gb300.h"

int main()
{
    std::string in((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
    char* out = nullptr;
    char* log = nullptr;
    int rc = ft_run_json(in.c_str(), &out, &log);
    if (log) {
        std::fputs(log, stderr);
        ft_free(log);
    }
    if (rc != FT_OK || !out) {
        if (out) ft_free(out);
        return rc ? rc : 1;
    }
    std::printf("%s\n", out);
    ft_free(out);
    return 0;
}
