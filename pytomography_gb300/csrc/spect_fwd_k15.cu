// PSF forward projector instance for the 15-tap bucket (spect_fwd_psf.cuh).
#include "spect_fwd_psf.cuh"

namespace gb {

GB_FWD_PSF_INSTANCE(15)
GB_FWD2_INSTANCE(15)

}  // namespace gb
