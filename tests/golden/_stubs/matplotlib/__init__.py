"""Stand-in: the reference's Poisson tutorial imports pyplot and tri at module level."""
