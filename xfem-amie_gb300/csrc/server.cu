// server.cu -- continuous-batching solve server (see amie_gpu.h).
#include "internal.h"

using namespace amie;

extern "C" amie_status amie_server_start(amie_ctx *, const amie_server_config *, amie_server **out)
{
    if (out) *out = nullptr;
    set_error("server not available in this build");
    return AMIE_BAD_INPUT;
}
extern "C" amie_status amie_submit(amie_server *, const amie_request *, uint64_t *) { return AMIE_BAD_INPUT; }
extern "C" amie_status amie_poll(amie_server *, uint64_t, amie_result *, double *) { return AMIE_BAD_INPUT; }
extern "C" amie_status amie_cancel(amie_server *, uint64_t) { return AMIE_BAD_INPUT; }
extern "C" amie_status amie_server_drain(amie_server *, double) { return AMIE_BAD_INPUT; }
extern "C" amie_status amie_server_stop(amie_server *) { return AMIE_OK; }
