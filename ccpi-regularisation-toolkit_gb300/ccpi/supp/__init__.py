"""Supporting utilities (synthetic phantoms) for the GB300 regularisers."""
