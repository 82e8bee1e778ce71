"""GB300-native two-site finite DMRG (drop-in for gqmps2's TwoSiteFiniteVMPS)."""
