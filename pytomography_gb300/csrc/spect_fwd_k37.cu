// PSF forward projector instance for the 37-tap bucket (spect_fwd_psf.cuh).
#include "spect_fwd_psf.cuh"

namespace gb {

GB_FWD_PSF_INSTANCE(37)

}  // namespace gb
