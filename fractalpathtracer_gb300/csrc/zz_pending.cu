#include "bridge_internal.h"
extern "C" {
int fpt_metal_diagnostic_render(const char *, const char *, const char *, size_t, const struct FptRenderConfig *, const struct FptDiagnosticConfig *, double *, char *error, size_t error_len) { fpt::set_error(error, error_len, "diagnostic: not built"); return 1; }
int fpt_test_typed_soa(const char *, const struct FptRenderConfig *, struct FptStitchValidationStats *, char *error, size_t error_len) { fpt::set_error(error, error_len, "typed soa: not built"); return 1; }
}
