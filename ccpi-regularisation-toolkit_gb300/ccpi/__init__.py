"""GB300-native drop-in for the CCPi Regularisation Toolkit's ``ccpi`` package."""
