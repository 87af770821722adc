"""nemaktis_gb300: GB300-native (sm_103a) z-stepping backend for Nemaktis' bpm-solver.

Modules:
  bpm_backend  drop-in for the reference's SWIG module (run_backend_without_mask/_with_mask)
  api          plans, batched multi-sample runs, timing
  microscope   objective focalisation and incoherent spectra of the output fields
                (OpticalFields / FieldViewer)
  workloads    seeded synthetic director fields and settings for the benchmark configurations
"""
__version__ = "0.1.0"
