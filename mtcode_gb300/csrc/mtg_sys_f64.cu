// mtg_sys_f64.cu -- double instantiation of the handle implementation.
#include "mtg_sys.cuh"

namespace mtg_impl {
SysBase *make_sys_f64(const mtg_config &cfg) { return new Sys<double>(cfg); }
}  // namespace mtg_impl
