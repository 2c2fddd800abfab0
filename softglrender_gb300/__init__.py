"""GB300-native (sm_103a) back-end for SoftGLRender's software rendering pipeline."""
