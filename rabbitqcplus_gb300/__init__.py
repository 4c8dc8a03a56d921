"""GB300-native CARE read error correction (the --correctWithCare path of RabbitQCPlus)."""
