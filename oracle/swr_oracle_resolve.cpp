// Oracle (test infrastructure, see swr_oracle.h): vis-buffer resolve.
#include "swr_oracle_common.h"

extern "C" void orc_resolve(orc_framebuffer*, const orc_shading_context*) {
    fprintf(stderr, "orc_resolve: not built yet\n");
    abort();
}
