// PSF forward projector instance for the 11-tap bucket (spect_fwd_psf.cuh).
#include "spect_fwd_psf.cuh"

namespace gb {

GB_FWD_PSF_INSTANCE(11)
GB_FWD2_INSTANCE(11)

}  // namespace gb
