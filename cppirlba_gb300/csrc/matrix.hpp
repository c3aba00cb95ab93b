// Host-side matrix handles shared by the engine, the batched form and the
// differentiation form: the device gather plans of a base matrix, the opaque
// C handle (a base matrix or a centre/scale decorator over one), and the
// decorator chain flattened for the fused kernels.
#pragma once

#include <memory>
#include <vector>

#include "host.hpp"

namespace irlba_gb300 {

struct DirPlan {
    DirPlanDev dev;
    DevBuf segptr, idx, val, block_seg;
    DevBuf code;   // dictionary codes of val (coded plans; val stays for the other kernels)
};

// A user-defined operator in place of the stored gather plans: its products are
// the caller's functions (device code on the engine's stream, or host code with
// the vectors copied around each call).
struct UserOperator {
    irlba_gb300_device_product device = nullptr;
    irlba_gb300_host_product host = nullptr;
    void* user = nullptr;
};

struct BaseMatrix {
    int64_t nrow = 0, ncol = 0;
    irlba_gb300_form form = IRLBA_GB300_FORM_FP64;
    bool store_f64 = true;
    DirPlan mul;  // rows = nrow, x = ncol
    DirPlan adj;  // rows = ncol, x = nrow
    DevBuf dict;  // the value dictionary shared by coded plans
    UserOperator op;
    bool is_operator() const { return op.device != nullptr || op.host != nullptr; }
};

}  // namespace irlba_gb300

struct irlba_gb300_matrix {
    int kind = 0;  // 0 base, 1 centre, 2 scale
    const irlba_gb300_matrix* inner = nullptr;
    std::shared_ptr<irlba_gb300::BaseMatrix> base;
    std::vector<double> vec;
    int column = 1, divide = 1;
    int64_t nrow = 0, ncol = 0;
    irlba_gb300_form form = IRLBA_GB300_FORM_FP64;
};

namespace irlba_gb300 {

// Decorator chain flattened for the fused kernels.
struct Chain {
    const BaseMatrix* base = nullptr;
    const std::vector<double>* center = nullptr;
    const std::vector<double>* scale = nullptr;
    int scale_column = 1, scale_divide = 1;
    int center_outer = 0;
    std::shared_ptr<BaseMatrix> owned;  // the chain operator below, when one was built
};

// A decorator chain the fused kernels do not cover (more than one
// CenteredMatrix or ScaledMatrix over the base, in any order) as a device
// operator whose products walk the chain (engine.cu); decos[0] is outermost.
std::shared_ptr<BaseMatrix> make_chain_operator(const BaseMatrix* base,
                                                const std::vector<const irlba_gb300_matrix*>& decos);

inline Chain flatten(const irlba_gb300_matrix* m) {
    std::vector<const irlba_gb300_matrix*> decos;
    const irlba_gb300_matrix* cur = m;
    while (cur && cur->kind != 0) {
        decos.push_back(cur);
        cur = cur->inner;
    }
    if (!cur) invalid("matrix handle has no base matrix");
    Chain ch;
    ch.base = cur->base.get();
    int ncenter = 0, nscale = 0;
    for (auto* d : decos) (d->kind == 1 ? ncenter : nscale)++;
    if (ncenter > 1 || nscale > 1) {
        ch.owned = make_chain_operator(ch.base, decos);
        ch.base = ch.owned.get();
        return ch;
    }
    for (auto* d : decos) {
        if (d->kind == 1) ch.center = &d->vec;
        else {
            ch.scale = &d->vec;
            ch.scale_column = d->column;
            ch.scale_divide = d->divide;
        }
    }
    // decos[0] is outermost.
    if (ncenter == 1 && nscale == 1) ch.center_outer = (decos[0]->kind == 1) ? 1 : 0;
    return ch;
}

// Paths that read the stored entries (column statistics, SpMM, SDDMM, the raw
// SpMV entry point) reject user-defined operators.
inline void require_stored(const BaseMatrix* b, const char* what) {
    if (b->is_operator())
        throw Error(IRLBA_GB300_ERROR_UNSUPPORTED,
                    std::string(what) + " needs a stored (sparse or dense) matrix, not a user-defined operator");
}

}  // namespace irlba_gb300
