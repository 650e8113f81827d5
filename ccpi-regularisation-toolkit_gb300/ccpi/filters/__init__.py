"""GB300 regularisers with the reference's ``ccpi.filters`` module layout."""
