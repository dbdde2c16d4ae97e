"""process_gb300 — GB300-native mutation placement and bulk-sequencing simulation
for ProCESS (drop-in for the RACES calls behind ``MutationEngine$place_mutations``
and ``simulate_seq``)."""
from ._lib import DomainError, ProcessError, UnsupportedError, device_count
from .engine import (CNA, SNV, WGD, BasicIlluminaSequencer, Batch, ErrorlessIlluminaSequencer, GenomeSpec, Mutation,
                     MutationEngine, PhylogeneticForest, SampledCell, SamplesForest, SBS_CLASSES, ID_CLASSES, load_passenger_CNAs,
                     load_phylogenetic_forest,
                     driver_regions, read_signature_table, sequence_counts, simulate_normal_seq, simulate_seq)

__all__ = [
    "Batch", "CNA", "SNV", "WGD", "BasicIlluminaSequencer", "ErrorlessIlluminaSequencer", "GenomeSpec", "Mutation",
    "MutationEngine", "PhylogeneticForest", "SampledCell", "SamplesForest", "SBS_CLASSES", "ID_CLASSES", "load_passenger_CNAs", "load_phylogenetic_forest",
    "driver_regions", "read_signature_table", "sequence_counts",
    "simulate_normal_seq", "simulate_seq", "DomainError", "ProcessError", "UnsupportedError", "device_count",
]
