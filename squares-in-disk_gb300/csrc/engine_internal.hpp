// Internal (non-exported) accessors of the host engine for other translation units of libsid.
#pragma once

#include "../../include/sid.h"
#include "engine.cuh"

namespace sid {

/// What another translation unit needs to launch a registered lemma's kernels.
struct LemmaView {
    const LemmaKernels* kernels;
    int device;
    int nargs;
    int last_static_arg;            // -1 if the lemma has no static split
    int last_static_subdivisions;
};

/// Record `msg` as this thread's last error (copied into fixed storage; never allocates).
void internal_set_error(const char* msg);

/// Look up a registered lemma; SID_OK or SID_ERR_INVALID. Never allocates.
int internal_lemma_view(sid_engine* engine, int lemma_id, LemmaView* out);

} // namespace sid
