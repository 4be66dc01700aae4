"""GB300-native finite-temperature AFQMC sweep for ALF.

Modules:
  sweep        Chains: the Python mirror of the C ABI (include/alfgpu.h) over batched chains
  model        Ham_Set equivalents: hopping exponentials and interaction vertices
  rng          the counter-based draw stream shared by the device and the host
  bins         scalar observable bins, walker / rank reduction, legacy *_scal files
  lattice_obs  lattice-resolved observables, legacy *_eq / *_tau files, ana_eq
  analysis     ALF's jackknife (errors_mod)
  replicas     one process per GPU: seeds and the whole-job time
Submodules are imported on use; importing the package loads no CUDA code.
"""
