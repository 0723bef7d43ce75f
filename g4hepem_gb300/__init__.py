"""GB300-native G4HepEmRun stepping physics.

The C-ABI is include/g4hepem_gb300.h (library: libg4hepem_gb300.so, built by
g4hepem_gb300.build); `native` is its Python front end, `workload` builds the
benchmark track batches, `tables.synth` writes synthetic G4HepEmState tables.
"""
__all__ = ["build", "native", "workload"]
