"""
sa_gb300 -- GB300-native multi-emitter Levenberg-Marquardt localisation
engine for storm-analysis (3D-DAOSTORM Gaussian models and Spliner).

Modules:
  loadclib     loads libsa_cuda.so (the CUDA engine) and declares its C ABI
  dao_fit_c    MultiFitter classes (reference sa_library/dao_fit_c.py)
  cubic_fit_c  CSplineFit classes (reference spliner/cubic_fit_c.py)
  engine       BatchFitter: many frames per launch
  serving      continuous-batching request loop
  synth        seeded synthetic workloads of the benchmark configurations
  build        compiles the engine for sm_103a
"""
