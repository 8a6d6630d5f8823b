"""The CPU oracle (test infrastructure only): C restatements of the
reference's NEMOLite2D step and tracer-advection iteration, the recipe that
compiles the reference's own PSy layers, and their Python loaders
(``oracle.cpu``).  Nothing in the GPU product imports this package."""
