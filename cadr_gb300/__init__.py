"""cadr_gb300: GB300-native (sm_103a) drawable-processing pass of CadR."""
