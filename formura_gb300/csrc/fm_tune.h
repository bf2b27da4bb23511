// fm_tune.h — process-wide tuning knobs (kernel variant, tile/chunk sizes).
//
// Every knob has an automatic default; fm_tune_set (C ABI) overrides it, which
// the autotuner and the variant-coverage tests use.  Knobs never change
// results: every variant of a kernel is bit-exact with the others.
#pragma once

namespace fm {
int tune_get(const char *key, int fallback);
}
