"""GB300-native Lienard-Wiechert field integration for TEUFEL observers."""
