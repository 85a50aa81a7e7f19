"""GB300-native rebuild of the se2wave explicit spectral-element time loop."""
