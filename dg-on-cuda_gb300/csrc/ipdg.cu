// ipdg.cu -- matrix-free laplace_2d (IPDG) apply and preconditioned CG.
#include "dgc_internal.hpp"

namespace dgc {

struct IpdgState {};

int ipdg_init(dgc_handle_s* h) {
  (void)h;
  return DGC_OK;
}

void ipdg_free(dgc_handle_s* h) {
  delete h->ipdg;
  h->ipdg = nullptr;
}

void ipdg_operators_changed(dgc_handle_s* h) { (void)h; }

}  // namespace dgc
