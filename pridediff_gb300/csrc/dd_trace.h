// NVTX ranges around the library's entry points (host side only), so that a
// profiler's timeline shows each operator, plan and data-consistency step by
// name.  NVTX3 is header-only; without a profiler attached a range costs a
// branch.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace ddtrace {

// Names of the operator codes (DD_OP_*) and scan types (DD_SCAN_* / DD_SCAN3_*).
inline const char *op_name(int op) {
    static const char *n[] = {"Proj", "ProjTrans", "BackProj", "BackProjTrans", "BackProjWeighted",
                              "BackProjTransWeighted"};
    return (op >= 0 && op < 6) ? n[op] : "op?";
}

struct Range {
    explicit Range(const char *what) { nvtxRangePushA(what); }
    Range(const char *what, int scan, int op, bool three_d) {
        static const char *s2[] = {"para", "fan-flat", "fan-arc"};
        static const char *s3[] = {"cone-flat", "cone-arc", "spiral"};
        const char *sc = (scan >= 0 && scan < 3) ? (three_d ? s3[scan] : s2[scan]) : "scan?";
        char buf[96];
        int k = 0;
        for (const char *p = what; *p && k < 40; p++) buf[k++] = *p;
        buf[k++] = ' ';
        if (op >= 0) {   // plans and data-consistency steps name no operator
            for (const char *p = op_name(op); *p && k < 80; p++) buf[k++] = *p;
            buf[k++] = ' ';
        }
        for (const char *p = sc; *p && k < 94; p++) buf[k++] = *p;
        buf[k] = 0;
        nvtxRangePushA(buf);
    }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

}   // namespace ddtrace
