"""GB300-native (sm_103a) backend for vkhr's volumetric level-of-detail path."""
