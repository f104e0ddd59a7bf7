// NVTX ranges on the host threads that plan and launch the stages, so that a
// profiler can select a stage or a kernel kind (ncu --nvtx --nvtx-include
// "damascus@Vec/" ...).  NVTX is header-only and costs a branch when no tool is
// attached.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace dm {

inline nvtxDomainHandle_t nvtx_domain() {
    static nvtxDomainHandle_t d = nvtxDomainCreateA("damascus");
    return d;
}

class NvtxRange {
   public:
    explicit NvtxRange(const char* name) {
        nvtxEventAttributes_t a = {};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(nvtx_domain(), &a);
    }
    ~NvtxRange() { nvtxDomainRangePop(nvtx_domain()); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

inline const char* stage_name(int stage) {
    static const char* const names[] = {"Init", "Vec", "Poly", "Done", "Failed"};
    return stage >= 0 && stage < 5 ? names[stage] : "?";
}

}  // namespace dm
