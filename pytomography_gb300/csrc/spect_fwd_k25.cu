// PSF forward projector instance for the 25-tap bucket (spect_fwd_psf.cuh).
#include "spect_fwd_psf.cuh"

namespace gb {

GB_FWD_PSF_INSTANCE(25)
GB_FWD2_INSTANCE(25)

}  // namespace gb
