// PSF forward projector instance for the 29-tap bucket (spect_fwd_psf.cuh).
#include "spect_fwd_psf.cuh"

namespace gb {

GB_FWD_PSF_INSTANCE(29)
GB_FWD2_INSTANCE(29)

}  // namespace gb
