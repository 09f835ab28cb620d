"""GB300-native photon propagation for neutrino telescopes.

The photon-propagation hot path of chrhck/NeutrinoTelescopes (Julia +
CUDA.jl) rebuilt as hand-written sm_103a CUDA behind the C ABI of
include/ntp.h (libntp.so); this package is the host side, mirroring the
reference's names: PhotonPropSetup, propagate_photons,
make_hits_from_photons, calc_total_weight, calc_time_residual, the emitters,
targets, media and spectra.
"""
from . import _abi
from .detection import (DetectionSphere, MultiPMTDetector, PMTWavelengthAcceptance, area_acceptance,
                        get_pmt_count, make_detector_cube, make_detector_hex, make_pom_pmt_coordinates,
                        make_targets, p_one_pmt_acc, string_of_modules)
from .lightyield import (AxiconeEmitter, CherenkovTrackEmitter, ExtendedCherenkovEmitter, LongitudinalParameters,
                         LongitudinalParameterisation, Particle, PEMinus, PEPlus, PGamma, PencilEmitter,
                         PointlikeCherenkovEmitter, PointlikeIsotropicEmitter, PointlikeTimeRangeEmitter,
                         cherenkov_ang_dist, cherenkov_track_length, longitudinal_profile, oversample_source,
                         split_source, total_lightyield)
from .medium import (MediumProperties, SimpleWater, WaterProperties, make_cascadia_medium_properties,
                     make_simple_water)
from .photon_prop import (HitTable, PhotonHit, PhotonPropSetup, calc_time_residual, calc_total_weight,
                          make_hits_from_photons, pmt_summary, propagate_photons, resample_simulation)
from .spectrum import (CherenkovSpectrum, InverseSquareSpectrum, Monochromatic, frank_tamm, frank_tamm_inverted_cdf,
                       frank_tamm_norm)

__all__ = [n for n in dir() if not n.startswith("_")]
