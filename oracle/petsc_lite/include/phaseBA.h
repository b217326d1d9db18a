/* fvmic2d optional phase model header: not part of the marker path (COMPBA is undefined) */
