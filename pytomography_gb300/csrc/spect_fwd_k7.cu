// PSF forward projector instance for the 7-tap bucket (spect_fwd_psf.cuh).
#include "spect_fwd_psf.cuh"

namespace gb {

GB_FWD_PSF_INSTANCE(7)
GB_FWD2_INSTANCE(7)

}  // namespace gb
