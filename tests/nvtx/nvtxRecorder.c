/* Test-only NVTX injection library: loaded by NVTX through NVTX_INJECTION64_PATH, it takes the
 * push and pop slots of NVTX's core table and writes each range's name (and each pop) to the file
 * named by ARTF_NVTX_LOG. */
#include <nvtx3/nvToolsExt.h>

#include <stdio.h>
#include <stdlib.h>

static FILE* logFile;

static int NVTX_API recordPush(const char* name) {
    if (logFile) fprintf(logFile, "push %s\n", name), fflush(logFile);
    return 0;
}

static int NVTX_API recordPop(void) {
    if (logFile) fprintf(logFile, "pop\n"), fflush(logFile);
    return 0;
}

int InitializeInjectionNvtx2(NvtxGetExportTableFunc_t getExportTable) {
    const NvtxExportTableCallbacks* callbacks =
        (const NvtxExportTableCallbacks*)getExportTable(NVTX_ETID_CALLBACKS);
    NvtxFunctionTable table = 0;
    unsigned int size = 0;
    if (!callbacks || !callbacks->GetModuleFunctionTable(NVTX_CB_MODULE_CORE, &table, &size)) return 0;
    if (size <= NVTX_CBID_CORE_RangePop) return 0;
    *table[NVTX_CBID_CORE_RangePushA] = (NvtxFunctionPointer)recordPush;
    *table[NVTX_CBID_CORE_RangePop] = (NvtxFunctionPointer)recordPop;
    const char* path = getenv("ARTF_NVTX_LOG");
    logFile = path ? fopen(path, "w") : 0;
    return 1;
}
