"""HTTP front end (FastAPI) with the reference's ``/api/ppr`` contract."""
