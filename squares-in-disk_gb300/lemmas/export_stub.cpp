// Engine stand-in linked only into the lemma IR exporter: with SID_EXPORT_DIR set, run_prover never
// reaches the engine, so every entry point here just reports that no engine is present.
#include "sid.h"
extern "C" {
void sid_prove_opts_default(sid_prove_opts* o){ *o = sid_prove_opts{}; }
const char* sid_last_error(void){ return "lemma exporter build: no engine linked"; }
int sid_engine_create(int, sid_engine**){ return SID_ERR_UNSUPPORTED; }
void sid_engine_destroy(sid_engine*){}
int sid_lemma_register(sid_engine*, const char*, size_t, int*){ return SID_ERR_UNSUPPORTED; }
int sid_lemma_info(sid_engine*, int, int*, uint64_t*){ return SID_ERR_UNSUPPORTED; }
int sid_lemma_root_box(sid_engine*, int, double*){ return SID_ERR_UNSUPPORTED; }
int sid_prove(sid_engine*, int, const sid_prove_opts*, sid_result*){ return SID_ERR_UNSUPPORTED; }
int sid_fetch_criticals(sid_engine*, int, double*, uint64_t, uint64_t*){ return SID_ERR_UNSUPPORTED; }
int sid_eval_batch(sid_engine*, int, const double*, const double*, uint64_t, double*, double*, int8_t*){ return SID_ERR_UNSUPPORTED; }
int sid_eval_batch_device(sid_engine*, int, const double*, const double*, uint64_t, double*, double*, int8_t*, void*){ return SID_ERR_UNSUPPORTED; }
}
