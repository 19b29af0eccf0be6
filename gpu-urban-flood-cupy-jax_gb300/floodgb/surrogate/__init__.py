"""Learned surrogate: a message-passing network on the triangle dual graph,
trained on trajectories of the FV solver, screening rainfall ensembles for
hourly depth and maximum depth; the solver re-runs flagged and audited
members and judges the surrogate's error."""
