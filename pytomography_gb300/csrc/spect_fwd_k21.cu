// PSF forward projector instance for the 21-tap bucket (spect_fwd_psf.cuh).
#include "spect_fwd_psf.cuh"

namespace gb {

GB_FWD_PSF_INSTANCE(21)
GB_FWD2_INSTANCE(21)

}  // namespace gb
