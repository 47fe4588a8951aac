"""IO mirrors of ``src/pytomography/io`` for the data formats either side of the projector
path (scanner geometry, listmode -> sinogram binning)."""
