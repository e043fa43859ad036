"""GB300-native implementation of GliomaUQ's Fisher-Kolmogorov block step and
imaging log-likelihood (host-side mirror over the C-ABI library libgbglioma)."""
