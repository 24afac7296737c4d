"""CPU oracle of vkhr's volumetric level-of-detail path (test infrastructure only)."""
