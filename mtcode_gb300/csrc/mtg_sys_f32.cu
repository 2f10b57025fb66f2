// mtg_sys_f32.cu -- float instantiation of the handle implementation.
#include "mtg_sys.cuh"

namespace mtg_impl {
SysBase *make_sys_f32(const mtg_config &cfg) { return new Sys<float>(cfg); }
}  // namespace mtg_impl
