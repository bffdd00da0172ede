/* Test helper: an NVTX injection library that writes every range push and
 * pop it sees to the file named by OGS_NVTX_LOG.  NVTX loads it from
 * NVTX_INJECTION64_PATH at the first NVTX call of the process and calls
 * InitializeInjectionNvtx2, which installs the two callbacks in the core
 * function table. */
#include <stdio.h>
#include <stdlib.h>

#include <nvtx3/nvToolsExt.h>

static FILE* out;

static int probe_push(const char* message) {
  if (out) {
    fprintf(out, "push %s\n", message ? message : "");
    fflush(out);
  }
  return 0;
}

static int probe_pop(void) {
  if (out) {
    fprintf(out, "pop\n");
    fflush(out);
  }
  return 0;
}

int InitializeInjectionNvtx2(NvtxGetExportTableFunc_t get_table) {
  const NvtxExportTableCallbacks* cb = (const NvtxExportTableCallbacks*)get_table(NVTX_ETID_CALLBACKS);
  NvtxFunctionTable table = 0;
  unsigned int size = 0;
  if (!cb || !cb->GetModuleFunctionTable(NVTX_CB_MODULE_CORE, &table, &size) || !table) return 0;
  if (size <= NVTX_CBID_CORE_RangePop) return 0;
  *table[NVTX_CBID_CORE_RangePushA] = (NvtxFunctionPointer)probe_push;
  *table[NVTX_CBID_CORE_RangePop] = (NvtxFunctionPointer)probe_pop;
  const char* path = getenv("OGS_NVTX_LOG");
  out = path ? fopen(path, "w") : NULL;
  return 1;
}
