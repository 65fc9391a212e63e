ArrayLike = object
