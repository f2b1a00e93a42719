"""nt_gb300.predict -- kernel-regression consumers (neural_tangents/_src/predict.py)."""
