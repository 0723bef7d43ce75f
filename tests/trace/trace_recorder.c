/* trace_recorder.c -- an NVTX injection library for the tests: loaded by
 * the NVTX calls of libg4hepem_gb300.so when NVTX_INJECTION64_PATH names it,
 * it appends one line per domain range push or pop to the file that
 * HEPEM_TRACE_LOG names:
 *
 *   push <domain> <message> <int64 payload>
 *   pop <domain>
 *
 * It subscribes to the CORE2 (domain) callbacks only, through the export
 * table that the NVTX headers define (nvtx3/nvtxDetail/nvtxTypes.h). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <nvtx3/nvToolsExt.h>

struct recorder_domain {
  char name[64];
};

static FILE* g_log = NULL;

static const char* domain_name(nvtxDomainHandle_t d) {
  return d ? ((const struct recorder_domain*)(const void*)d)->name : "(default)";
}

static nvtxDomainHandle_t NVTX_API on_domain_create(const char* name) {
  struct recorder_domain* d = (struct recorder_domain*)calloc(1, sizeof(*d));
  if (!d) return NULL;
  snprintf(d->name, sizeof(d->name), "%s", name ? name : "");
  return (nvtxDomainHandle_t)(void*)d;
}

static int NVTX_API on_push(nvtxDomainHandle_t d, const nvtxEventAttributes_t* a) {
  const char* msg = (a && a->messageType == NVTX_MESSAGE_TYPE_ASCII && a->message.ascii) ? a->message.ascii : "?";
  const long long payload = (a && a->payloadType == NVTX_PAYLOAD_TYPE_INT64) ? a->payload.llValue : -1;
  if (g_log) {
    fprintf(g_log, "push %s %s %lld\n", domain_name(d), msg, payload);
    fflush(g_log);
  }
  return 0;
}

static int NVTX_API on_pop(nvtxDomainHandle_t d) {
  if (g_log) {
    fprintf(g_log, "pop %s\n", domain_name(d));
    fflush(g_log);
  }
  return 0;
}

int InitializeInjectionNvtx2(NvtxGetExportTableFunc_t get_table) {
  const char* path = getenv("HEPEM_TRACE_LOG");
  if (!path || !get_table) return 0;
  g_log = fopen(path, "a");
  if (!g_log) return 0;
  const NvtxExportTableCallbacks* cb = (const NvtxExportTableCallbacks*)get_table(NVTX_ETID_CALLBACKS);
  NvtxFunctionTable table = NULL;
  unsigned int size = 0;
  if (!cb || !cb->GetModuleFunctionTable || !cb->GetModuleFunctionTable(NVTX_CB_MODULE_CORE2, &table, &size) ||
      !table || size < NVTX_CBID_CORE2_DomainCreateA)
    return 0;
  *table[NVTX_CBID_CORE2_DomainCreateA] = (NvtxFunctionPointer)on_domain_create;
  *table[NVTX_CBID_CORE2_DomainRangePushEx] = (NvtxFunctionPointer)on_push;
  *table[NVTX_CBID_CORE2_DomainRangePop] = (NvtxFunctionPointer)on_pop;
  return 1;
}
