"""sunaengine_gb300 — SunaEngine's deterministic Q16.16 PBF substep on one GB300."""
