"""CPU oracles of the hot path and loaders of Etalon's own kernels: test and bench infrastructure
only (the checker, never the thing measured or shipped); the product never imports this package."""
