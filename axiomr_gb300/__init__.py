"""AxiomR-GB300: the AxiomR software-rasterisation draw path on one GB300 (sm_103a)."""
